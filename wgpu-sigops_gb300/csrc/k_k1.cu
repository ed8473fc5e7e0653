// Plain k1 recovery kernel instantiation (separate translation unit so
// the per-curve kernels compile in parallel).
#include "plain.cuh"

namespace sg {

cudaError_t launch_plain_k1(const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* gtab, uint8_t* out, uint8_t* status,
                             uint32_t* err, int grid, cudaStream_t stream) {
  ecdsa_plain_kernel<K1Traits><<<grid, PLAIN_BLOCK, 0, stream>>>(sigs, msgs, n, gtab, out, status, err);
  return cudaGetLastError();
}

int occupancy_plain_k1() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ecdsa_plain_kernel<K1Traits>, PLAIN_BLOCK, 0);
  return b;
}

}  // namespace sg
