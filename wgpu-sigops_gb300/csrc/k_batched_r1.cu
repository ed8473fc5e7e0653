// Single-curve batched kernels for P-256 recovery: configurations 0..3 (launch
// shapes at the default window widths) and the simultaneous-inversion kernels
// around the curve kernel; configurations 4..7 are in k_batched_r1_w.cu
// (one translation unit each, so that they compile in parallel).
#include "batched.cuh"

namespace sg {

int batched_occupancy_r1_w(int config);
cudaError_t batched_curve_r1_w(int config, const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, const DeferBufs& d,
                                  uint32_t* err, cudaStream_t stream);

int batched_occupancy_r1(int config) {
  switch (config) {
    case 0: return CurveKernel<1, 0>::occupancy();
    case 1: return CurveKernel<1, 1>::occupancy();
    case 2: return CurveKernel<1, 2>::occupancy();
    case 3: return CurveKernel<1, 3>::occupancy();
    default: return batched_occupancy_r1_w(config);
  }
}

// the curve's part of a single-curve step, on one stream
cudaError_t batched_launch_r1(int config, const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, const DeferBufs& d,
                              uint32_t* err, cudaStream_t stream) {
  launch_rinv<1>(io, idx, sc, d, stream);
  cudaError_t e;
  switch (config) {
    case 0: e = CurveKernel<1, 0>::launch(io, idx, t, sc, d, err, stream); break;
    case 1: e = CurveKernel<1, 1>::launch(io, idx, t, sc, d, err, stream); break;
    case 2: e = CurveKernel<1, 2>::launch(io, idx, t, sc, d, err, stream); break;
    case 3: e = CurveKernel<1, 3>::launch(io, idx, t, sc, d, err, stream); break;
    default: e = batched_curve_r1_w(config, io, idx, t, sc, d, err, stream); break;
  }
  if (e != cudaSuccess) return e;
  launch_finish<1>(io, idx, sc, d, stream);
  return cudaGetLastError();
}

}  // namespace sg
