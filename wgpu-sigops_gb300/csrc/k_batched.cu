// Batched mixed-curve engine: classify kernel, variant dispatch.
#include "batched.cuh"

namespace sg {

__global__ void classify_kernel(const uint8_t* __restrict__ curves, size_t n, uint32_t* __restrict__ idx, Scratch* sc) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const unsigned lane = threadIdx.x & 31u;
  for (size_t base = (size_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    size_t i = base + threadIdx.x;
    int c = i < n ? curves[i] : -1;
    if (c > 2) c = -1;  // unknown tags are skipped (host validates)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      unsigned m = __ballot_sync(0xffffffffu, c == k);
      if (!m) continue;
      uint32_t off = 0;
      int leader = __ffs(m) - 1;
      if ((int)lane == leader) off = atomicAdd(&sc->count[k], (uint32_t)__popc(m));
      off = __shfl_sync(0xffffffffu, off, leader);
      if (c == k) idx[(size_t)k * n + off + __popc(m & ((1u << lane) - 1u))] = (uint32_t)i;
    }
  }
}

int batched_occupancy_0();
int batched_occupancy_1();
int batched_occupancy_2();
int batched_occupancy_3();
cudaError_t batched_launch_0(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);
cudaError_t batched_launch_1(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);
cudaError_t batched_launch_2(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);
cudaError_t batched_launch_3(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);

// variants: 0 = 256 threads x 1 block/SM, 1 = 256 x 2, 2 = 128 x 4, 3 = 64 threads
static const int kBlock[BATCHED_VARIANTS] = {256, 256, 128, 64};

int batched_variant_block(int v) { return (v >= 0 && v < BATCHED_VARIANTS) ? kBlock[v] : 0; }

int batched_max_blocks_per_sm(int v) {
  switch (v) {
    case 0: return batched_occupancy_0();
    case 1: return batched_occupancy_1();
    case 2: return batched_occupancy_2();
    case 3: return batched_occupancy_3();
    default: return 0;
  }
}

cudaError_t launch_batched(const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, uint8_t* out,
                           uint8_t* status, uint32_t* idx, void* scratch, const uint32_t* gk1, const uint32_t* gr1, const uint32_t* ged,
                           uint32_t* err, int grid, int variant, int classify_grid, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  Scratch* sc = (Scratch*)scratch;
  cudaError_t e = cudaMemsetAsync(sc, 0, sizeof(Scratch), stream);
  if (e != cudaSuccess) return e;
  classify_kernel<<<classify_grid, 256, 0, stream>>>(curves, n, idx, sc);
  MixedIO io{curves, sigs, msgs, pks, out, status, n};
  BatchTables t{gk1, gr1, ged};
  switch (variant) {
    case 0: return batched_launch_0(io, idx, t, sc, err, grid, stream);
    case 1: return batched_launch_1(io, idx, t, sc, err, grid, stream);
    case 2: return batched_launch_2(io, idx, t, sc, err, grid, stream);
    case 3: return batched_launch_3(io, idx, t, sc, err, grid, stream);
    default: return cudaErrorInvalidValue;
  }
}

size_t batched_scratch_bytes() { return sizeof(Scratch); }

}  // namespace sg
