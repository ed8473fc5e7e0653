// Single-curve batched kernels for ed25519 verification at three occupancy levels:
// 0 = 256 threads x 1 block per SM (up to 255 registers), 1 = 128 x 3 (170),
// 2 = 256 x 2 (128), 3 = 64 threads with at most 200 registers (5 blocks per SM).
#include "batched.cuh"

namespace sg {

int batched_occupancy_ed(int level) {
  int b = 0;
  if (level == 0) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_kernel<256, 1, CM_ED>, 256, 0);
  else if (level == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_kernel<128, 3, CM_ED>, 128, 0);
  else if (level == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_kernel<256, 2, CM_ED>, 256, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_kernel_r<64, 200, CM_ED>, 64, 0);
  return b;
}

cudaError_t batched_launch_ed(int level, const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, uint32_t* err,
                              int grid, cudaStream_t stream) {
  if (level == 0) batched_kernel<256, 1, CM_ED><<<grid, 256, 0, stream>>>(io, idx, t, sc, err);
  else if (level == 1) batched_kernel<128, 3, CM_ED><<<grid, 128, 0, stream>>>(io, idx, t, sc, err);
  else if (level == 2) batched_kernel<256, 2, CM_ED><<<grid, 256, 0, stream>>>(io, idx, t, sc, err);
  else batched_kernel_r<64, 200, CM_ED><<<grid, 64, 0, stream>>>(io, idx, t, sc, err);
  return cudaGetLastError();
}

}  // namespace sg
