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
//      secp256k1 recovery with small spills.
// Generator-table entries are read from global memory (L2-resident) as the
// windows need them.
// Scratch (global memory beyond inputs and outputs): Scratch below.
#pragma once
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
};

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
// curve CURVE's index list; blocks past the list's end return at once.
template <int BLOCK, int CURVE>
__device__ __forceinline__ void curve_body(const MixedIO& io, const uint32_t* __restrict__ idx, const BatchTables& tabs, Scratch* sc,
                                           uint32_t* err) {
  const uint32_t cnt = sc->count[CURVE];
  const uint32_t first = blockIdx.x * BLOCK;
  if (first >= cnt) return;
  const uint32_t* tk1 = tabs.k1;  // G and 2^128 G multiples (GLV)
  const uint32_t* tr1 = tabs.r1;
  const uint32_t* ted = tabs.ed;
  const uint32_t slot = first + threadIdx.x;
  if (slot >= cnt) return;
  const size_t i = idx[(size_t)CURVE * io.n + slot];
  uint32_t s[16], m[8], o[16];
  load_words(io.sigs, i, 16, s);
  load_words(io.msgs, i, 8, m);
  uint8_t st;
  if constexpr (CURVE == 0) st = ecdsa_recover<K1Traits, true>(s, m, tk1, o);
  else if constexpr (CURVE == 1) st = ecdsa_recover<R1Traits>(s, m, tr1, o);
  else st = ed_item(io, i, s, m, ted, o);
  store_words(io.out, i, 16, o);
  io.status[i] = st;
}

// occupancy by blocks per SM ...
template <int BLOCK, int MINB, int CURVE>
__global__ void __launch_bounds__(BLOCK, MINB) batched_curve_kernel(MixedIO io, const uint32_t* __restrict__ idx, BatchTables tabs, Scratch* sc,
                                                                uint32_t* err) {
  curve_body<BLOCK, CURVE>(io, idx, tabs, sc, err);
}

// ... or by an explicit register cap
template <int BLOCK, int MAXREG, int CURVE>
__global__ void __launch_bounds__(BLOCK) __maxnreg__(MAXREG) batched_curve_kernel_r(MixedIO io, const uint32_t* __restrict__ idx,
                                                                                  BatchTables tabs, Scratch* sc, uint32_t* err) {
  curve_body<BLOCK, CURVE>(io, idx, tabs, sc, err);
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
