// Batched mixed-curve kernel, variant 2: 128 threads x 4 blocks per SM.
#include "batched.cuh"

namespace sg {

int batched_occupancy_2() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_kernel<128, 4, CM_ALL>, 128, 0);
  return b;
}

cudaError_t batched_launch_2(const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, uint32_t* err, int grid,
                               cudaStream_t stream) {
  batched_kernel<128, 4, CM_ALL><<<grid, 128, 0, stream>>>(io, idx, t, sc, err);
  return cudaGetLastError();
}

}  // namespace sg
