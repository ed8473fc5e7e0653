// Batched mixed-curve engine: classify kernel, variant dispatch.
#include <algorithm>
#include <atomic>

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
int batched_occupancy_k1(int config);
int batched_occupancy_r1(int config);
int batched_occupancy_ed(int config);
cudaError_t batched_launch_0(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);
cudaError_t batched_launch_1(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);
cudaError_t batched_launch_2(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);
cudaError_t batched_launch_3(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);
cudaError_t batched_launch_k1(int, const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, const DeferBufs&, uint32_t*, cudaStream_t);
cudaError_t batched_launch_r1(int, const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, const DeferBufs&, uint32_t*, cudaStream_t);
cudaError_t batched_launch_ed(int, const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, const DeferBufs&, uint32_t*, cudaStream_t);

static const int kFusedBlock[BATCHED_FUSED_VARIANTS] = {256, 256, 128, 256};  // 1, 2, 3: one tile per warp, no loop

int curve_config_block(int config) {
  static const int kBlock[CURVE_CONFIGS] = {256, 128, 256, 64, 512, 128, 256, 256};
  return config >= 0 && config < CURVE_CONFIGS ? kBlock[config] : 0;
}

void curve_config_windows(int config, int* wr, int* wg) {
  *wr = config == 5 ? 4 : config == 6 ? 6 : ECDSA_WR;
  *wg = config == 7 ? SMALL_WG : ECDSA_WG;
}

// blocks per SM of curve c's kernel in a configuration (queried once; the
// kernels are the same on every device of one process)
int curve_config_occupancy(int c, int config) {
  static std::atomic<int> cache[3][CURVE_CONFIGS];
  if (c < 0 || c > 2 || config < 0 || config >= CURVE_CONFIGS) return 0;
  int b = cache[c][config].load(std::memory_order_relaxed);
  if (b == 0) {
    b = c == 0 ? batched_occupancy_k1(config) : c == 1 ? batched_occupancy_r1(config) : batched_occupancy_ed(config);
    cache[c][config].store(b, std::memory_order_relaxed);
  }
  return b;
}

int batched_variant_block(int v) {
  if (v >= 0 && v < BATCHED_FUSED_VARIANTS) return kFusedBlock[v];
  return (v >= BATCHED_FUSED_VARIANTS && v < BATCHED_VARIANTS) ? 256 : 0;
}

int batched_max_blocks_per_sm(int v) {
  switch (v) {
    case 0: return batched_occupancy_0();
    case 1: return batched_occupancy_1();
    case 2: return batched_occupancy_2();
    case 3: return batched_occupancy_3();
    default: break;
  }
  if (v < BATCHED_FUSED_VARIANTS || v >= BATCHED_VARIANTS) return 0;
  // in 256-thread blocks: the grid cap of a single-curve variant
  int m = 0;
  for (int c = 0; c < 3; ++c) {
    const int cfg = split_config(v, c);
    const int b = (curve_config_occupancy(c, cfg) * curve_config_block(cfg) + 255) / 256;  // rounded up: never caps a kernel
    if (b <= 0) return 0;
    m = b > m ? b : m;
  }
  return m;
}

cudaError_t fork_streams_create(ForkStreams* f, int priority) {
  *f = ForkStreams{};
  cudaError_t e;
  for (int k = 0; k < 2; ++k)
    if ((e = cudaStreamCreateWithPriority(&f->aux[k], cudaStreamNonBlocking, priority)) != cudaSuccess) return e;
  for (int k = 0; k < 3; ++k)
    if ((e = cudaEventCreateWithFlags(&f->ev[k], cudaEventDisableTiming)) != cudaSuccess) return e;
  return cudaSuccess;
}

void fork_streams_destroy(ForkStreams* f) {
  for (int k = 0; k < 2; ++k)
    if (f->aux[k]) cudaStreamDestroy(f->aux[k]);
  for (int k = 0; k < 3; ++k)
    if (f->ev[k]) cudaEventDestroy(f->ev[k]);
  *f = ForkStreams{};
}

static cudaError_t launch_curve(int c, int config, const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc,
                                const DeferBufs& d, uint32_t* err, cudaStream_t s) {
  if (c == 0) return batched_launch_k1(config, io, idx, t, sc, d, err, s);
  if (c == 1) return batched_launch_r1(config, io, idx, t, sc, d, err, s);
  return batched_launch_ed(config, io, idx, t, sc, d, err, s);
}

cudaError_t launch_batched(const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, uint8_t* out,
                           uint8_t* status, uint32_t* idx, void* scratch, void* defer, const GenTables& tabs, uint32_t* err, int grid,
                           int variant, int classify_grid, const ForkStreams* fork, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  // the per-curve index lists hold 32-bit item indices; the single-curve
  // variants need the shared-inversion scratch
  if (variant < 0 || variant >= BATCHED_VARIANTS || grid <= 0 || n > 0xffffffffull) return cudaErrorInvalidValue;
  if (variant >= BATCHED_FUSED_VARIANTS && !defer) return cudaErrorInvalidValue;
  Scratch* sc = (Scratch*)scratch;
  cudaError_t e = cudaMemsetAsync(sc, 0, sizeof(Scratch), stream);
  if (e != cudaSuccess) return e;
  classify_kernel<<<classify_grid, 256, 0, stream>>>(curves, n, idx, sc);
  MixedIO io{curves, sigs, msgs, pks, out, status, n};
  BatchTables t{tabs.big[0], tabs.big[1], tabs.big[2], {tabs.small[0], tabs.small[1], tabs.small[2]}};
  switch (variant) {
    case 0: return batched_launch_0(io, idx, t, sc, err, grid, stream);
    case 1: return batched_launch_1(io, idx, t, sc, err, grid, stream);
    case 2: return batched_launch_2(io, idx, t, sc, err, grid, stream);
    case 3: return batched_launch_3(io, idx, t, sc, err, grid, stream);
    default: break;
  }
  // single-curve kernels: secp256k1 on the caller's stream, the other two on
  // the side streams, so that each starts filling SMs as another's blocks retire
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  cudaStream_t s[3] = {stream, stream, stream};
  if (fork) {
    if ((e = cudaEventRecord(fork->ev[0], stream)) != cudaSuccess) return e;
    for (int k = 0; k < 2; ++k) {
      if ((e = cudaStreamWaitEvent(fork->aux[k], fork->ev[0], 0)) != cudaSuccess) return e;
      s[k + 1] = fork->aux[k];
    }
  }
  cudaError_t first = cudaSuccess;
  const DeferBufs d{reinterpret_cast<uint4*>(defer), reinterpret_cast<uint4*>(defer) + 2 * n};
  for (int c = 0; c < 3; ++c) {
    // one item per thread: the kernel sizes its grid to the batch
    e = launch_curve(c, split_config(variant, c), io, idx, t, sc, d, err, s[c]);
    if (e != cudaSuccess && first == cudaSuccess) first = e;
  }
  if (fork) {  // join, even after a failed launch, so no side stream stays forked
    for (int k = 0; k < 2; ++k) {
      e = cudaEventRecord(fork->ev[k + 1], fork->aux[k]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, fork->ev[k + 1], 0);
      if (e != cudaSuccess && first == cudaSuccess) first = e;
    }
  }
  return first;
}

size_t batched_scratch_bytes() { return sizeof(Scratch); }
size_t batched_defer_bytes(size_t n) { return n * DEFER_BYTES_PER_ITEM; }

}  // namespace sg
