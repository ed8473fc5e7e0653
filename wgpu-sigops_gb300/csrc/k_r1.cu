// Plain r1 recovery kernel instantiations (one translation unit per curve
// so the kernels compile in parallel).  Variant v: 0 -> 256-thread blocks, one
// per SM (no register cap); 1 -> two per SM (128 registers); 2 -> 128-thread
// blocks, three per SM (170 registers).
#include "plain.cuh"

namespace sg {

cudaError_t launch_plain_r1(const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* gtab, uint8_t* out, uint8_t* status,
                             uint32_t* err, int variant, cudaStream_t stream) {
  const int block = plain_variant_block(variant);
  const unsigned grid = (unsigned)((n + block - 1) / block);
  if (variant == 1) ecdsa_plain_kernel<R1Traits, 256, 2><<<grid, 256, 0, stream>>>(sigs, msgs, n, gtab, out, status, err);
  else if (variant == 2) ecdsa_plain_kernel<R1Traits, 128, 3><<<grid, 128, 0, stream>>>(sigs, msgs, n, gtab, out, status, err);
  else ecdsa_plain_kernel<R1Traits, 256, 1><<<grid, 256, 0, stream>>>(sigs, msgs, n, gtab, out, status, err);
  return cudaGetLastError();
}

// a batch too small to fill the GPU: one warp per block, so the warps spread
// over the SMs (a lone warp runs a signature faster than eight sharing an SM)
cudaError_t launch_plain_r1_small(const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* gtab, uint8_t* out, uint8_t* status,
                                  uint32_t* err, cudaStream_t stream) {
  ecdsa_plain_kernel<R1Traits, 32, 1><<<(unsigned)((n + 31) / 32), 32, 0, stream>>>(sigs, msgs, n, gtab, out, status, err);
  return cudaGetLastError();
}

int occupancy_plain_r1(int variant) {
  int b = 0;
  if (variant == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ecdsa_plain_kernel<R1Traits, 256, 2>, 256, 0);
  else if (variant == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ecdsa_plain_kernel<R1Traits, 128, 3>, 128, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ecdsa_plain_kernel<R1Traits, 256, 1>, 256, 0);
  return b;
}

}  // namespace sg
