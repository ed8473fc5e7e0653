// Batched mixed-curve engine: verifies a batch that mixes secp256k1 recovery,
// P-256 recovery and ed25519 verification.
//
// The reference runs one curve per call and pads every batch to a power of two
// (src/secp256k1_ecdsa.rs:25-44); it has no mixed-curve path.  Here:
//   1. classify_kernel buckets item indices by curve (warp-aggregated atomics
//      into per-curve index lists);
//   2. either the fused batched_kernel, a persistent grid in which each warp
//      repeatedly takes the next 32-item tile from a global counter (tiles
//      never straddle curves, so the curve dispatch is warp-uniform and no
//      lane idles on another curve's code), registers sized for the largest
//      path;
//   3. or three single-curve kernels (batched_curve_kernel), one item per
//      thread and no loop, each with its own register budget, launched side
//      by side on forked streams.  With no loop state live across the
//      signature arithmetic, the 168-register budget (12 warps per SM) fits
//      secp256k1 recovery with small spills.  These share work across
//      items that a one-signature-per-thread kernel cannot: the inversions of
//      r mod n (before) and of the result point's Z mod p (after) run as
//      simultaneous inversions over INV_BATCH items per thread (Montgomery's
//      trick: three multiplications per item and one inversion per batch),
//      in rinv_kernel and finish_kernel around the curve kernel.
// Generator-table entries are read from global memory (L2-resident) as the
// windows need them.
// Scratch (global memory beyond inputs and outputs): Scratch and the per-curve
// index lists; the single-curve path also DeferBufs (128 bytes per item).
#pragma once
#include <type_traits>

#include "kernels.cuh"

namespace sg {

constexpr int BATCH_TILE = 32;  // items per warp work unit

// curve masks of batched_kernel
constexpr int CM_K1 = 1, CM_R1 = 2, CM_ED = 4, CM_ALL = 7;

struct Scratch {
  uint32_t count[3];   // items per curve (classify)
  uint32_t next_tile;  // work-stealing counter of the fused kernel
  uint32_t pad[4];     // keeps the record at 32 bytes
};

// Mixed output record: ECDSA key bytes, or for ed25519 byte 0 = valid.
struct MixedIO {
  const uint8_t* curves;  // n tags (0/1/2)
  const uint8_t* sigs;    // n*64
  const uint8_t* msgs;    // n*32
  const uint8_t* pks;     // n*32 (read for ed25519 items only)
  uint8_t* out;           // n*64
  uint8_t* status;        // n
  size_t n;
};

struct BatchTables {
  const uint32_t* k1;
  const uint32_t* r1;
  const uint32_t* ed;
  const uint32_t* small[3];  // 8-bit-window tables (staged into shared memory)
};

// Item-indexed scratch of the single-curve path's shared inversions
struct DeferBufs {
  uint4* rinv;  // n x 32 bytes: r^-1 mod n (Montgomery form) of each ECDSA item
  uint4* pt;    // n x 96 bytes: X, Y, Z of each item's result point, awaiting Z^-1
};
constexpr size_t DEFER_BYTES_PER_ITEM = 128;
constexpr int INV_BATCH = 16;  // items per thread of a simultaneous inversion
constexpr int INV_BLOCK = 128;

__device__ __forceinline__ u256 ld_u256(const uint4* p) {
  const uint4 a = p[0], b = p[1];
  return u256{{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w}};
}
__device__ __forceinline__ void st_u256(uint4* p, const u256& v) {
  p[0] = make_uint4(v.w[0], v.w[1], v.w[2], v.w[3]);
  p[1] = make_uint4(v.w[4], v.w[5], v.w[6], v.w[7]);
}

// ed25519 item of a batch: out byte 0 = valid, the rest zero
__device__ __forceinline__ uint8_t ed_item(const MixedIO& io, size_t i, const uint32_t s[16], const uint32_t m[8], const uint32_t* ted,
                                           uint32_t o[16]) {
  uint32_t p[8];
  load_words(io.pks, i, 8, p);
  const uint8_t st = ed25519_verify(s, m, p, ted);
#pragma unroll
  for (int k = 0; k < 16; ++k) o[k] = 0;
  o[0] = st == ST_OK;
  return st;
}

// One item: load, verify or recover, store.  Called rather than inlined, so
// that the tile loop's pointers and counters are saved once per signature
// instead of staying live (about 20 registers) through its arithmetic.
template <int CURVE>
__device__ __noinline__ void batched_item(const MixedIO io, size_t i, const uint32_t* tab) {
  uint32_t s[16], m[8], o[16];
  load_words(io.sigs, i, 16, s);
  load_words(io.msgs, i, 8, m);
  uint8_t st;
  if constexpr (CURVE == 0) st = ecdsa_recover<K1Traits, true>(s, m, tab, o);
  else if constexpr (CURVE == 1) st = ecdsa_recover<R1Traits>(s, m, tab, o);
  else st = ed_item(io, i, s, m, tab, o);
  store_words(io.out, i, 16, o);
  io.status[i] = st;
}

template <int CM>
__device__ __forceinline__ void batched_body(const MixedIO& io, const uint32_t* __restrict__ idx, const BatchTables& tabs, Scratch* sc,
                                             uint32_t* err) {
  const uint32_t* tk1 = tabs.k1;  // G and 2^128 G multiples (GLV)
  const uint32_t* tr1 = tabs.r1;
  const uint32_t* ted = tabs.ed;

  const uint32_t n1 = (CM & CM_K1) ? sc->count[0] : 0, n2 = (CM & CM_R1) ? sc->count[1] : 0, n3 = (CM & CM_ED) ? sc->count[2] : 0;
  const uint32_t t1 = (n1 + BATCH_TILE - 1) / BATCH_TILE, t2 = (n2 + BATCH_TILE - 1) / BATCH_TILE, t3 = (n3 + BATCH_TILE - 1) / BATCH_TILE;
  const uint32_t total = t1 + t2 + t3;
  uint32_t* counter = &sc->next_tile;
  const unsigned lane = threadIdx.x & 31u;
  for (;;) {
    uint32_t tile = 0;
    if (lane == 0) tile = atomicAdd(counter, 1u);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= total) break;
    int curve;
    uint32_t first, cnt;
    if (tile < t1) { curve = 0; first = tile * BATCH_TILE; cnt = n1; }
    else if (tile < t1 + t2) { curve = 1; first = (tile - t1) * BATCH_TILE; cnt = n2; }
    else { curve = 2; first = (tile - t1 - t2) * BATCH_TILE; cnt = n3; }
    const uint32_t slot = first + lane;
    if (slot < cnt) {
      const size_t i = idx[(size_t)curve * io.n + slot];
      if constexpr (CM == CM_K1) {
        batched_item<0>(io, i, tk1);
      } else if constexpr (CM == CM_R1) {
        batched_item<1>(io, i, tr1);
      } else if constexpr (CM == CM_ED) {
        batched_item<2>(io, i, ted);
      } else {
        static_assert(CM == CM_ALL, "one curve or all three");
        if (curve == 0) batched_item<0>(io, i, tk1);
        else if (curve == 1) batched_item<1>(io, i, tr1);
        else batched_item<2>(io, i, ted);
      }
    }
  }
}

// the fused kernel (CM_ALL): occupancy by blocks per SM
template <int BLOCK, int MINB, int CM>
__global__ void __launch_bounds__(BLOCK, MINB) batched_kernel(MixedIO io, const uint32_t* __restrict__ idx, BatchTables tabs, Scratch* sc,
                                                        uint32_t* err) {
  batched_body<CM>(io, idx, tabs, sc, err);
}


// Single-curve kernel body: block b serves items [b BLOCK, (b + 1) BLOCK) of
// curve CURVE's index list; blocks past the list's end return at once.  The
// result point stays projective: an item whose checks pass stores X, Y, Z in
// d.pt for finish_kernel (status ST_OK = pending there); any other item gets
// its final status and a zero record here.  ECDSA items take r^-1 from
// d.rinv (rinv_kernel).  With 8-bit generator windows (WG = SMALL_WG) the
// block first stages its curve's 128-entry table into shared memory.
template <int BLOCK, int CURVE, int WR, int WG>
__device__ __forceinline__ void curve_body(const MixedIO& io, const uint32_t* __restrict__ idx, const BatchTables& tabs, Scratch* sc,
                                           const DeferBufs& d, uint32_t* err) {
  const uint32_t cnt = sc->count[CURVE];
  const uint32_t first = blockIdx.x * BLOCK;
  if (first >= cnt) return;
  const uint32_t* tab = CURVE == 0 ? tabs.k1 : CURVE == 1 ? tabs.r1 : tabs.ed;
  if constexpr (WG == SMALL_WG) {
    // the block's copy of the 8-bit-window table (secp256k1: G and 2^128 G halves)
    constexpr uint32_t WORDS = CURVE == 0 ? 2 * SMALL_GTAB * 16 : CURVE == 1 ? SMALL_GTAB * 16 : SMALL_GTAB * 24;
    __shared__ __align__(128) uint32_t stab[WORDS];
    __shared__ __align__(8) uint64_t bar;
    if (!stage_to_smem(stab, tabs.small[CURVE], WORDS * 4u, &bar, err)) return;
    tab = stab;
  }
  const uint32_t slot = first + threadIdx.x;
  if (slot >= cnt) return;
  const size_t i = idx[(size_t)CURVE * io.n + slot];
  uint32_t s[16], m[8];
  load_words(io.sigs, i, 16, s);
  load_words(io.msgs, i, 8, m);
  uint8_t st;
  u256 X, Y, Z;
  if constexpr (CURVE < 2) {
    using T = typename std::conditional<CURVE == 0, K1Traits, R1Traits>::type;
    u256 r, sv, z;
    APoint R;
    JPoint Q;
    st = ecdsa_prepare<T>(s, m, r, sv, z, R);
    if (st == ST_OK) st = ecdsa_key_jacobian<T, CURVE == 0, WR, WG>(sv, z, R, ld_u256(d.rinv + 2 * i), tab, Q);
    X = Q.X;
    Y = Q.Y;
    Z = Q.Z;
  } else {
    uint32_t p[8];
    load_words(io.pks, i, 8, p);
    EPoint Rp;
    st = ed25519_point<WR, WG>(s, m, p, tab, Rp);
    X = Rp.X;
    Y = Rp.Y;
    Z = Rp.Z;
  }
  if (st == ST_OK) {
    st_u256(d.pt + 6 * i, X);
    st_u256(d.pt + 6 * i + 2, Y);
    st_u256(d.pt + 6 * i + 4, Z);
  } else {
    uint32_t o[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) o[k] = 0;
    store_words(io.out, i, 16, o);
  }
  io.status[i] = st;
}

// Threads of a simultaneous-inversion kernel over curve CURVE's list: thread t
// takes slots t, t + T, t + 2T, ... (T = ceil(count / INV_BATCH)), at most
// INV_BATCH of them
__device__ __forceinline__ bool inv_thread(const Scratch* sc, int curve, uint32_t& t, uint32_t& T, uint32_t& cnt) {
  cnt = sc->count[curve];
  T = (cnt + INV_BATCH - 1) / INV_BATCH;
  t = blockIdx.x * blockDim.x + threadIdx.x;
  return t < T;
}

// r^-1 mod n of every ECDSA item of curve CURVE (0 secp256k1, 1 P-256), by one
// simultaneous inversion per thread, into d.rinv
template <int CURVE>
__global__ void __launch_bounds__(INV_BLOCK) rinv_kernel(MixedIO io, const uint32_t* __restrict__ idx, Scratch* sc, DeferBufs d) {
  using T = typename std::conditional<CURVE == 0, K1Traits, R1Traits>::type;
  using S = typename T::S;
  uint32_t t, nt, cnt;
  if (!inv_thread(sc, CURVE, t, nt, cnt)) return;
  u256 v[INV_BATCH], pre[INV_BATCH];
  uint32_t item[INV_BATCH];
  int m = 0;
#pragma unroll 1
  for (; m < INV_BATCH; ++m) {
    const uint32_t slot = t + (uint32_t)m * nt;
    if (slot >= cnt) break;
    item[m] = idx[(size_t)CURVE * io.n + slot];
    uint32_t s[16];
    load_words(io.sigs, item[m], 16, s);
    v[m] = ecdsa_r_factor<T>(s);
  }
  batch_invert<S>(v, pre, m, [](const u256& x) { return S::from_int(S::inv_int(S::to_int(x))); });
#pragma unroll 1
  for (int j = 0; j < m; ++j) st_u256(d.rinv + 2 * (size_t)item[j], v[j]);
}

// The pending items of curve CURVE after its curve kernel: one simultaneous
// inversion of their Z per thread, then the affine key's bytes (ECDSA) or the
// encoding's comparison with the R bytes (ed25519)
template <int CURVE>
__global__ void __launch_bounds__(INV_BLOCK) finish_kernel(MixedIO io, const uint32_t* __restrict__ idx, Scratch* sc, DeferBufs d) {
  uint32_t t, nt, cnt;
  if (!inv_thread(sc, CURVE, t, nt, cnt)) return;
  u256 v[INV_BATCH], pre[INV_BATCH];
  uint32_t item[INV_BATCH];
  int m = 0;
#pragma unroll 1
  for (int j = 0; j < INV_BATCH; ++j) {
    const uint32_t slot = t + (uint32_t)j * nt;
    if (slot >= cnt) break;
    const uint32_t i = idx[(size_t)CURVE * io.n + slot];
    if (io.status[i] != ST_OK) continue;  // final already
    item[m] = i;
    v[m] = ld_u256(d.pt + 6 * (size_t)i + 4);
    ++m;
  }
  if (m == 0) return;
  if constexpr (CURVE < 2) {
    using T = typename std::conditional<CURVE == 0, K1Traits, R1Traits>::type;
    using F = typename T::F;
    batch_invert<F>(v, pre, m, [](const u256& x) { return F::inv(x); });
#pragma unroll 1
    for (int j = 0; j < m; ++j) {
      const size_t i = item[j];
      JPoint Q;
      Q.X = ld_u256(d.pt + 6 * i);
      Q.Y = ld_u256(d.pt + 6 * i + 2);
      uint32_t o[16];
      ecdsa_encode_key<T>(Q, v[j], o);
      store_words(io.out, i, 16, o);
    }
  } else {
    batch_invert<FpEd>(v, pre, m, [](const u256& x) { return FpEd::inv(x); });
#pragma unroll 1
    for (int j = 0; j < m; ++j) {
      const size_t i = item[j];
      EPoint Rp;
      Rp.X = ld_u256(d.pt + 6 * i);
      Rp.Y = ld_u256(d.pt + 6 * i + 2);
      uint32_t s[16], o[16];
      load_words(io.sigs, i, 16, s);
      const uint8_t st = ed25519_compare(Rp, v[j], s);
#pragma unroll
      for (int k = 0; k < 16; ++k) o[k] = 0;
      o[0] = st == ST_OK;
      store_words(io.out, i, 16, o);
      io.status[i] = st;
    }
  }
}

// occupancy by blocks per SM ...
template <int BLOCK, int MINB, int CURVE, int WR = ECDSA_WR, int WG = ECDSA_WG>
__global__ void __launch_bounds__(BLOCK, MINB) batched_curve_kernel(MixedIO io, const uint32_t* __restrict__ idx, BatchTables tabs, Scratch* sc,
                                                                DeferBufs d, uint32_t* err) {
  curve_body<BLOCK, CURVE, WR, WG>(io, idx, tabs, sc, d, err);
}

// ... or by an explicit register cap
template <int BLOCK, int MAXREG, int CURVE>
__global__ void __launch_bounds__(BLOCK) __maxnreg__(MAXREG) batched_curve_kernel_r(MixedIO io, const uint32_t* __restrict__ idx,
                                                                                  BatchTables tabs, Scratch* sc, DeferBufs d, uint32_t* err) {
  curve_body<BLOCK, CURVE, ECDSA_WR, ECDSA_WG>(io, idx, tabs, sc, d, err);
}

// The single-curve kernels in configuration CFG (launch.h lists them): block
// shape / register budget and window widths.  Configurations 0..3 are
// compiled with the simultaneous-inversion kernels in k_batched_<curve>.cu,
// 4..7 in k_batched_<curve>_w.cu.
template <int CURVE, int CFG>
struct CurveKernel {
  static constexpr int BLOCK = CFG == 1 || CFG == 5 ? 128 : CFG == 3 ? 64 : CFG == 4 ? 512 : 256;
  static constexpr int WR = CFG == 5 ? 4 : CFG == 6 ? 6 : ECDSA_WR;
  static constexpr int WG = CFG == 7 ? SMALL_WG : ECDSA_WG;
  static auto fn() {
    if constexpr (CFG == 0) return batched_curve_kernel<256, 1, CURVE>;
    else if constexpr (CFG == 1) return batched_curve_kernel<128, 3, CURVE>;
    else if constexpr (CFG == 3) return batched_curve_kernel_r<64, 144, CURVE>;
    else if constexpr (CFG == 4) return batched_curve_kernel<512, 1, CURVE>;
    else if constexpr (CFG == 5) return batched_curve_kernel<128, 3, CURVE, WR, WG>;
    else return batched_curve_kernel<256, 2, CURVE, WR, WG>;  // 2, 6, 7
  }
  static int occupancy() {
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn(), BLOCK, 0);
    return b;
  }
  static cudaError_t launch(const MixedIO& io, const uint32_t* idx, const BatchTables& t, Scratch* sc, const DeferBufs& d, uint32_t* err,
                            cudaStream_t stream) {
    const unsigned grid = (unsigned)((io.n + BLOCK - 1) / BLOCK);
    fn()<<<grid, BLOCK, 0, stream>>>(io, idx, t, sc, d, err);
    return cudaGetLastError();
  }
};

// r^-1 by simultaneous inversion (ECDSA curves), before the curve kernel
template <int CURVE>
void launch_rinv(const MixedIO& io, const uint32_t* idx, Scratch* sc, const DeferBufs& d, cudaStream_t stream) {
  const unsigned inv_grid = (unsigned)(((io.n + INV_BATCH - 1) / INV_BATCH + INV_BLOCK - 1) / INV_BLOCK);
  rinv_kernel<CURVE><<<inv_grid, INV_BLOCK, 0, stream>>>(io, idx, sc, d);
}

// the result points' Z^-1 by simultaneous inversion, after the curve kernel
template <int CURVE>
void launch_finish(const MixedIO& io, const uint32_t* idx, Scratch* sc, const DeferBufs& d, cudaStream_t stream) {
  const unsigned inv_grid = (unsigned)(((io.n + INV_BATCH - 1) / INV_BATCH + INV_BLOCK - 1) / INV_BLOCK);
  finish_kernel<CURVE><<<inv_grid, INV_BLOCK, 0, stream>>>(io, idx, sc, d);
}

// Fused kernel, one tile per warp: warp w of the grid takes tile w of the
// concatenated per-curve tile lists (no loop), so the curve dispatch stays
// warp-uniform and almost no state is live across the per-item call.
template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) batched_fused_flat_kernel(MixedIO io, const uint32_t* __restrict__ idx, BatchTables tabs,
                                                                     Scratch* sc, uint32_t* err) {
  const uint32_t n1 = sc->count[0], n2 = sc->count[1], n3 = sc->count[2];
  const uint32_t t1 = (n1 + BATCH_TILE - 1) / BATCH_TILE, t2 = (n2 + BATCH_TILE - 1) / BATCH_TILE, t3 = (n3 + BATCH_TILE - 1) / BATCH_TILE;
  const uint32_t first_tile = blockIdx.x * (BLOCK / 32);
  if (first_tile >= t1 + t2 + t3) return;
  const uint32_t* tk1 = tabs.k1;  // G and 2^128 G multiples (GLV)
  const uint32_t* tr1 = tabs.r1;
  const uint32_t* ted = tabs.ed;
  const uint32_t tile = first_tile + (threadIdx.x >> 5), lane = threadIdx.x & 31u;
  uint32_t slot;
  if (tile < t1) {
    slot = tile * BATCH_TILE + lane;
    if (slot < n1) batched_item<0>(io, idx[slot], tk1);
  } else if (tile < t1 + t2) {
    slot = (tile - t1) * BATCH_TILE + lane;
    if (slot < n2) batched_item<1>(io, idx[io.n + slot], tr1);
  } else if (tile < t1 + t2 + t3) {
    slot = (tile - t1 - t2) * BATCH_TILE + lane;
    if (slot < n3) batched_item<2>(io, idx[2 * io.n + slot], ted);
  }
}

}  // namespace sg
