// Batched mixed-curve kernel, variant 0: 256 threads x 1 blocks per SM.
#include "batched.cuh"

namespace sg {

int batched_occupancy_0() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_kernel<256, 1, CM_ALL>, 256, 0);
  return b;
}

cudaError_t batched_launch_0(const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, uint32_t* err, int grid,
                               cudaStream_t stream) {
  batched_kernel<256, 1, CM_ALL><<<grid, 256, 0, stream>>>(io, idx, t, sc, err);
  return cudaGetLastError();
}

}  // namespace sg
