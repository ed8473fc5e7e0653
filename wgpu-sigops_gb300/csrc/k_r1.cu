// Plain r1 recovery kernel instantiations (one translation unit per curve
// so the kernels compile in parallel).  Variant v: v = 0 -> one block of
// PLAIN_BLOCK threads per SM (no register cap), v = 1 -> two (128 registers).
#include "plain.cuh"

namespace sg {

cudaError_t launch_plain_r1(const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* gtab, uint8_t* out, uint8_t* status,
                             uint32_t* err, int grid, int variant, cudaStream_t stream) {
  if (variant == 1)
    ecdsa_plain_kernel<R1Traits, 2><<<grid, PLAIN_BLOCK, 0, stream>>>(sigs, msgs, n, gtab, out, status, err);
  else
    ecdsa_plain_kernel<R1Traits, 1><<<grid, PLAIN_BLOCK, 0, stream>>>(sigs, msgs, n, gtab, out, status, err);
  return cudaGetLastError();
}

int occupancy_plain_r1(int variant) {
  int b = 0;
  if (variant == 1)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ecdsa_plain_kernel<R1Traits, 2>, PLAIN_BLOCK, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ecdsa_plain_kernel<R1Traits, 1>, PLAIN_BLOCK, 0);
  return b;
}

}  // namespace sg
