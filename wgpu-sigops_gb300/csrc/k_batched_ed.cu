// Single-curve batched kernels for ed25519 verification, one item per thread, at four
// occupancy levels: 0 = 256 threads x 1 block per SM (up to 255 registers),
// 1 = 128 x 3 (170), 2 = 256 x 2 (128), 3 = 64 threads with at most 144
// registers.  The grid covers the whole batch; blocks past the curve's item
// count return at once.
#include "batched.cuh"

namespace sg {

int batched_occupancy_ed(int level) {
  int b = 0;
  if (level == 0) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_curve_kernel<256, 1, 2>, 256, 0);
  else if (level == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_curve_kernel<128, 3, 2>, 128, 0);
  else if (level == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_curve_kernel<256, 2, 2>, 256, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_curve_kernel_r<64, 144, 2>, 64, 0);
  return b;
}

cudaError_t batched_launch_ed(int level, const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, uint32_t* err,
                              cudaStream_t stream) {
  const int block = level == 3 ? 64 : level == 1 ? 128 : 256;
  const unsigned grid = (unsigned)((io.n + block - 1) / block);
  if (level == 0) batched_curve_kernel<256, 1, 2><<<grid, 256, 0, stream>>>(io, idx, t, sc, err);
  else if (level == 1) batched_curve_kernel<128, 3, 2><<<grid, 128, 0, stream>>>(io, idx, t, sc, err);
  else if (level == 2) batched_curve_kernel<256, 2, 2><<<grid, 256, 0, stream>>>(io, idx, t, sc, err);
  else batched_curve_kernel_r<64, 144, 2><<<grid, 64, 0, stream>>>(io, idx, t, sc, err);
  return cudaGetLastError();
}

}  // namespace sg
