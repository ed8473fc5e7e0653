// Single-curve batched kernels for P-256 recovery, configurations 4..7: 512-thread
// blocks, 128 x 3 blocks with 4-bit per-point windows, and 256 x 2 blocks with
// 6-bit per-point windows or 8-bit generator windows whose table each block
// stages into shared memory.
#include "batched.cuh"

namespace sg {

int batched_occupancy_r1_w(int config) {
  switch (config) {
    case 4: return CurveKernel<1, 4>::occupancy();
    case 5: return CurveKernel<1, 5>::occupancy();
    case 6: return CurveKernel<1, 6>::occupancy();
    case 7: return CurveKernel<1, 7>::occupancy();
    default: return 0;
  }
}

cudaError_t batched_curve_r1_w(int config, const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, const DeferBufs& d,
                                  uint32_t* err, cudaStream_t stream) {
  switch (config) {
    case 4: return CurveKernel<1, 4>::launch(io, idx, t, sc, d, err, stream);
    case 5: return CurveKernel<1, 5>::launch(io, idx, t, sc, d, err, stream);
    case 6: return CurveKernel<1, 6>::launch(io, idx, t, sc, d, err, stream);
    case 7: return CurveKernel<1, 7>::launch(io, idx, t, sc, d, err, stream);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sg
