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
int batched_occupancy_k1(int level);
int batched_occupancy_r1(int level);
int batched_occupancy_ed(int level);
cudaError_t batched_launch_0(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);
cudaError_t batched_launch_1(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);
cudaError_t batched_launch_2(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);
cudaError_t batched_launch_3(const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, int, cudaStream_t);
cudaError_t batched_launch_k1(int, const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, cudaStream_t);
cudaError_t batched_launch_r1(int, const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, cudaStream_t);
cudaError_t batched_launch_ed(int, const MixedIO&, const uint32_t*, const BatchTables&, Scratch*, uint32_t*, cudaStream_t);

static const int kFusedBlock[BATCHED_FUSED_VARIANTS] = {256, 256, 128, 256};  // 1, 2, 3: one tile per warp, no loop

// single-curve kernels: occupancy level 0 = 256 threads x 1 block per SM,
// 1 = 128 x 3, 2 = 256 x 2 (8, 12 and 16 warps per SM), 3 = 64 threads with
// at most 144 registers (14 warps per SM)
constexpr int kLevels = 4;
static const int kLevelBlock[kLevels] = {256, 128, 256, 64};

// blocks per SM of curve c's single-curve kernel at an occupancy level
// (queried once; the kernels are the same on every device of one process)
static int curve_occupancy(int c, int level) {
  static std::atomic<int> cache[3][kLevels];
  int b = cache[c][level].load(std::memory_order_relaxed);
  if (b == 0) {
    b = c == 0 ? batched_occupancy_k1(level) : c == 1 ? batched_occupancy_r1(level) : batched_occupancy_ed(level);
    cache[c][level].store(b, std::memory_order_relaxed);
  }
  return b;
}

// variant 4 + a + 4 b + 16 c: levels a, b, c for secp256k1, P-256, ed25519
static int split_level(int variant, int c) {
  int v = variant - BATCHED_FUSED_VARIANTS;
  for (int k = 0; k < c; ++k) v /= kLevels;
  return v % kLevels;
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
    const int l = split_level(v, c);
    const int b = (curve_occupancy(c, l) * kLevelBlock[l] + 255) / 256;  // rounded up: never caps a kernel
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

static cudaError_t launch_curve(int c, int level, const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc,
                                uint32_t* err, cudaStream_t s) {
  if (c == 0) return batched_launch_k1(level, io, idx, t, sc, err, s);
  if (c == 1) return batched_launch_r1(level, io, idx, t, sc, err, s);
  return batched_launch_ed(level, io, idx, t, sc, err, s);
}

cudaError_t launch_batched(const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, uint8_t* out,
                           uint8_t* status, uint32_t* idx, void* scratch, const uint32_t* gk1, const uint32_t* gr1, const uint32_t* ged,
                           uint32_t* err, int grid, int variant, int classify_grid, const ForkStreams* fork, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  // the per-curve index lists hold 32-bit item indices
  if (variant < 0 || variant >= BATCHED_VARIANTS || grid <= 0 || n > 0xffffffffull) return cudaErrorInvalidValue;
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
  for (int c = 0; c < 3; ++c) {
    // one item per thread: the kernel sizes its grid to the batch
    e = launch_curve(c, split_level(variant, c), io, idx, t, sc, err, s[c]);
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

}  // namespace sg
