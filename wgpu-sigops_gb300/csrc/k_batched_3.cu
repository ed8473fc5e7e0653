// Batched mixed-curve kernel, variant 3: 64 threads x 1 block per SM (more fit by occupancy).
#include "batched.cuh"

namespace sg {

int batched_occupancy_3() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_kernel<64, 1, CM_ALL>, 64, 0);
  return b;
}

cudaError_t batched_launch_3(const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, uint32_t* err, int grid,
                               cudaStream_t stream) {
  batched_kernel<64, 1, CM_ALL><<<grid, 64, 0, stream>>>(io, idx, t, sc, err);
  return cudaGetLastError();
}

}  // namespace sg
