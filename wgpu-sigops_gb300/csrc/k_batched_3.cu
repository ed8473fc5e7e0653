// Batched mixed-curve kernel, variant 3: the fused kernel at 256 threads x 2 blocks per SM (128 registers, 16 warps per SM), one tile per warp, no loop.
#include "batched.cuh"

namespace sg {

int batched_occupancy_3() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_fused_flat_kernel<256, 2>, 256, 0);
  return b;
}

// the grid covers every tile of the batch (one per warp): at most n / 32 + 3 tiles
cudaError_t batched_launch_3(const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, uint32_t* err, int,
                               cudaStream_t stream) {
  const size_t tiles = (io.n + BATCH_TILE - 1) / BATCH_TILE + 3;
  const unsigned grid = (unsigned)((tiles + 256 / 32 - 1) / (256 / 32));
  batched_fused_flat_kernel<256, 2><<<grid, 256, 0, stream>>>(io, idx, t, sc, err);
  return cudaGetLastError();
}

}  // namespace sg
