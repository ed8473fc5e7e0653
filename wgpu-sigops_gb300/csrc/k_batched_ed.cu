// Single-curve batched kernels for ed25519 verification: configurations 0..3 (launch
// shapes at the default window widths) and the simultaneous-inversion kernels
// around the curve kernel; configurations 4..7 are in k_batched_ed_w.cu
// (one translation unit each, so that they compile in parallel).
#include "batched.cuh"

namespace sg {

int batched_occupancy_ed_w(int config);
cudaError_t batched_curve_ed_w(int config, const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, const DeferBufs& d,
                                  uint32_t* err, cudaStream_t stream);

int batched_occupancy_ed(int config) {
  switch (config) {
    case 0: return CurveKernel<2, 0>::occupancy();
    case 1: return CurveKernel<2, 1>::occupancy();
    case 2: return CurveKernel<2, 2>::occupancy();
    case 3: return CurveKernel<2, 3>::occupancy();
    default: return batched_occupancy_ed_w(config);
  }
}

// the curve's part of a single-curve step, on one stream
cudaError_t batched_launch_ed(int config, const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, const DeferBufs& d,
                              uint32_t* err, cudaStream_t stream) {
  cudaError_t e;
  switch (config) {
    case 0: e = CurveKernel<2, 0>::launch(io, idx, t, sc, d, err, stream); break;
    case 1: e = CurveKernel<2, 1>::launch(io, idx, t, sc, d, err, stream); break;
    case 2: e = CurveKernel<2, 2>::launch(io, idx, t, sc, d, err, stream); break;
    case 3: e = CurveKernel<2, 3>::launch(io, idx, t, sc, d, err, stream); break;
    default: e = batched_curve_ed_w(config, io, idx, t, sc, d, err, stream); break;
  }
  if (e != cudaSuccess) return e;
  launch_finish<2>(io, idx, sc, d, stream);
  return cudaGetLastError();
}

}  // namespace sg
