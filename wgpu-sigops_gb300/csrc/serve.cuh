// Device side of the serving loop: one persistent kernel that takes work from
// a pinned, mapped request ring on the host through a device-resident tile
// ring.
//
// No counterpart in the reference (each call there builds a device and runs one
// batch, src/gpu.rs:5-35).
//
//   host (sigops_server_submit)          device (serve_kernel)
//   ---------------------------          ---------------------
//   copies a request's items into the    feeder warp (block 0, warp 0): polls
//   pinned item ring grouped by curve,   the host's tile tail, copies new tiles
//   writes its 32-item single-curve      into three device-resident rings, one
//   tiles into the pinned tile ring,     per curve, 32 per round (one per
//   then publishes the host tile tail    lane), publishes their tails
//   (release)                            (release), and every 100 us moves
//                                        TPCs to a curve whose backlog needs
//                                        them
//                                        consumer warps (all others): claim the
//                                        next tile of their TPC's curve, read
//                                        its items from the pinned rings in
//                                        whole lines into shared memory,
//                                        verify them, write the
//                                        results back in whole lines; the warp
//                                        whose tile completes a request
//                                        appends it to the pinned completion
//                                        ring (release, system scope)
//
// The feeder does no per-request work (the host cut the tiles), so it keeps up
// although it shares an SM with compute-bound warps.  Host memory is only
// touched in whole, coalesced lines: a lane reading its own 64-byte signature
// and writing its own record would cost some 25 small transactions per item
// across the chip-to-chip link, and those, not the arithmetic, would bound
// the rate.
//
// The two SMs of a TPC work on one curve at a time: each curve's code is
// large, and SMs of one TPC running different curves thrash the instruction
// fetch path they share (a mixed stream of requests ran at a third of the
// single-curve rate with no affinity, and 15-25% slower per tile with the
// curve kept per SM instead of per TPC).  A TPC changes curve when its own
// curve has nothing left for it and its warps are all done (serve_next) or
// when the feeder moves it to a curve whose backlog needs it (serve_balance);
// a moved TPC finishes the tiles its warps hold.  Within a curve, tiles are
// claimed in the order they were published.
//
// A slot of a device ring is reused only after the request owning its
// previous tile has completed (the host reclaims ring space in submission
// order, and a curve's ring is as large as the host's), so every tile copied
// has been read.  Each tile carries its request's completion target: the
// running item count of its request slot after the request, so a slot's
// counter never needs resetting (requests reuse a slot only after the previous
// one completed).
//
// Every wait is bounded.  The feeder stops copying and sets `closing` when the
// host asks (stop), after idle_ns without a new tile, or after life_ns; a
// consumer leaves once closing is set and every ring is empty, so every
// published tile is processed before the kernel exits.  A consumer that finds
// no tile for longer than its poll budget without closing (a feeder that
// stopped) sets DEV_ERR_QUEUE_TIMEOUT and leaves; the host then fails the
// requests left unfinished instead of waiting for them forever.
#pragma once
#include "batched.cuh"

namespace sg {

// the host-visible control block (pinned, mapped)
struct ServeCtl {
  uint64_t tile_tail;  // tiles published (host)
  uint64_t tiles_fed;  // tiles copied into the device ring (feeder)
  uint32_t stop;       // host: close the kernel
  uint32_t err;        // device error bits of the serving kernel
  uint32_t exited;     // the launch number of the last kernel whose warps have all left
  uint32_t pad;
};

struct ServeTile {
  uint32_t shape;   // request slot | items (1..32) << 16 | curve << 24
  uint32_t first;   // first item of the tile in the item rings
  uint32_t seq;     // the request's sequence number (its low 16 bits go into the completion entry)
  uint32_t target;  // the slot's running item count once the request is complete
};

// device-resident queue state (kept across launches)
constexpr int SERVE_MODE_SLOTS = 256;   // curve assignment slots, indexed by %smid / SERVE_SMS_PER_SLOT modulo this
constexpr uint32_t SERVE_SMS_PER_SLOT = 2;  // the two SMs of a TPC work on one curve
struct ServeDev {
  uint64_t fed;           // tiles of the host ring copied (feeder)
  uint64_t ring_tail[3];  // tiles published in each curve's device ring (feeder)
  uint64_t ring_head[3];  // tiles claimed from each curve's ring (consumers)
  uint64_t comp_tail;     // completion entries written
  uint32_t closing;       // the feeder publishes no more tiles in this launch
  uint32_t live_warps;    // warps of this launch still running
  uint32_t mode[SERVE_MODE_SLOTS];  // the curve each slot (TPC) works on
  uint32_t busy[SERVE_MODE_SLOTS];  // warps of each slot holding a tile (or claiming one)
  uint32_t seen[SERVE_MODE_SLOTS];  // 1 for the slots the kernel runs on
  // kernel counters: tiles and items done, warp time working on tiles and
  // looking for one (globaltimer ns, summed over warps)
  unsigned long long tiles_done, items_done, work_ns, idle_ns;
  unsigned long long moves, drains;  // SM curve changes: by the feeder, by an SM with nothing left
};

// A completion entry: bits 0-31 the entry's position + 1 (how the host tells
// a new entry from the previous lap's), 32-47 the request slot, 48-63 the low
// 16 bits of the request's sequence number.
__host__ __device__ constexpr uint64_t serve_completion(uint64_t pos, uint32_t slot, uint32_t seq) {
  return (uint64_t)(uint32_t)(pos + 1) | ((uint64_t)(slot & 0xffffu) << 32) | ((uint64_t)(seq & 0xffffu) << 48);
}

struct ServeArgs {
  ServeCtl* ctl;              // pinned, mapped
  const ServeTile* htiles;    // tile_cap tiles (pinned, mapped), written by the host
  uint64_t* comp;             // R completion entries (pinned, mapped), a ring
  const uint8_t* sig;         // C items each (pinned, mapped): signatures, messages, keys
  const uint8_t* msg;
  const uint8_t* pk;
  uint8_t* out;               // C x 64 result records, C status bytes (pinned, mapped)
  uint8_t* st;
  ServeDev* dev;              // device memory
  ServeTile* tiles;           // three rings of tile_cap tiles (a power of two), one per curve
  uint32_t* count;            // R running item counts, one per request slot
  uint32_t R, C, tile_cap;
  BatchTables tabs;
  uint64_t idle_ns, life_ns;  // feeder: close after this long without a tile / in all
  uint32_t warps_per_sm;      // consumer warps an SM holds (a round of tiles)
  uint32_t warp_cap;          // tiles a TPC works on at once while its curve has no backlog
  uint32_t launch;            // this launch's number (ServeCtl::exited)
};

constexpr uint32_t SERVE_FEED_MAX_ITERS = 1u << 26;  // feeder polls per launch (bounds the loop; time limits end it first)
constexpr uint32_t SERVE_WAIT_MAX_POLLS = 1u << 21;  // consumer polls for one tile (about 4 s with the back-off)
constexpr uint64_t SERVE_BALANCE_NS = 100000;       // the feeder balances the curves' TPCs this often

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ uint64_t ld_acquire_sys_u64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_acquire_sys_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t ld_acquire_gpu_u64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_acquire_gpu_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu_u64(uint64_t* p, uint64_t v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_release_gpu_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release_sys_u64(uint64_t* p, uint64_t v) {
  asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_release_sys_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// 16 bytes of the host rings, coherent at system scope (the rings are reused)
__device__ __forceinline__ uint4 ld_sys_v4(const void* p) {
  uint4 v;
  asm volatile("ld.relaxed.sys.global.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p) : "memory");
  return v;
}

// A warp's staging area: 32 items x 32 words (signature 0-15, message 16-23,
// key 24-31); a result record replaces its item's signature words.  Items are
// read from and written to the pinned rings as consecutive 16-byte chunks
// (lane + 32 j: whole 128-byte lines), one load in flight per lane: the
// forms that keep several host-memory loads in flight per lane (all of a
// lane's loads issued before its stores, weak loads the compiler batches,
// loads exchanged by shuffles) each doubled a lone request's latency and made
// a tile 20% slower under load (measured).
constexpr int SERVE_STAGE_WORDS = 32 * 32;

// One item of a served request
template <int CURVE>
__device__ __noinline__ uint32_t serve_item(const uint32_t* s, const uint32_t* m, const uint32_t* p, const uint32_t* tab, uint32_t* o) {
  uint8_t st;
  if constexpr (CURVE == 0) {
    st = ecdsa_recover<K1Traits, true>(s, m, tab, o);
  } else if constexpr (CURVE == 1) {
    st = ecdsa_recover<R1Traits>(s, m, tab, o);
  } else {
    st = ed25519_verify(s, m, p, tab);
#pragma unroll
    for (int k = 0; k < 16; ++k) o[k] = 0;
    o[0] = st == ST_OK;
  }
  return st;
}

__device__ __forceinline__ uint32_t smid() {
  uint32_t v;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(v));
  return v;
}

__device__ __forceinline__ uint32_t warp_sum(uint32_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// The feeder warp's TPC assignment, every SERVE_BALANCE_NS.  A curve's
// pressure is its tiles waiting x the time a tile of it takes, per TPC
// working on it.  When the highest pressure exceeds twice the lowest plus one
// round of tiles (a tile per warp of a TPC), an eighth of the low-pressure
// curve's TPCs (at least one, idle ones first) move to the high-pressure
// curve; every curve keeps at least one TPC.  Together with the rule in
// serve_next (a TPC whose ring is empty and whose warps are all done moves to
// the curve with the most tiles waiting) the TPCs follow the mix within a
// millisecond, while a TPC changes curve only when the backlog asks for it:
// every move runs two curves on one TPC for up to a tile's time.
__device__ __forceinline__ void serve_balance(const ServeArgs& a, unsigned lane, const uint64_t tail[3]) {
  constexpr uint64_t kCost[3] = {100, 140, 90};  // relative time of a tile: secp256k1 (GLV), P-256, ed25519
  constexpr int PER = SERVE_MODE_SLOTS / 32;
  const uint32_t below = (1u << lane) - 1u;
  uint32_t md[PER], bz[PER];
  uint32_t n[3] = {0, 0, 0};
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const uint32_t sl = lane + 32 * j;
    md[j] = 3;
    bz[j] = 0;
    if (*(volatile uint32_t*)&a.dev->seen[sl]) {
      md[j] = min(*(volatile uint32_t*)&a.dev->mode[sl], 2u);
      bz[j] = *(volatile uint32_t*)&a.dev->busy[sl];
      n[md[j]] += 1;
    }
  }
  uint64_t w[3], p[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    n[k] = warp_sum(n[k]);
    const uint64_t head = *(volatile uint64_t*)&a.dev->ring_head[k];
    w[k] = tail[k] > head ? tail[k] - head : 0;
    p[k] = w[k] * kCost[k] * 64 / max(n[k], 1u);
  }
  int hi = -1, lo = -1;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (w[k] && (hi < 0 || p[k] > p[hi])) hi = k;
  }
  if (hi < 0) return;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (k != hi && n[k] > 1 && (lo < 0 || p[k] < p[lo])) lo = k;
  }
  if (lo < 0) return;
  const uint64_t round = kCost[hi] * 64 * a.warps_per_sm * SERVE_SMS_PER_SLOT;
  if (n[hi] > 0 && p[hi] <= 2 * p[lo] + round) return;
  const uint32_t m = min(max(n[lo] / 8, 1u), n[lo] - 1);
  // the first m slots of curve lo in slot order, idle ones first
  uint32_t moved = 0;
#pragma unroll 1
  for (int pass = 0; pass < 2 && moved < m; ++pass) {
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const bool cand = md[j] == (uint32_t)lo && (pass == 1 || bz[j] == 0);
      const uint32_t mask = __ballot_sync(0xffffffffu, cand);
      if (cand && moved + __popc(mask & below) < m) {
        *(volatile uint32_t*)&a.dev->mode[lane + 32 * j] = (uint32_t)hi;
        md[j] = (uint32_t)hi;
        atomicAdd(&a.dev->moves, 1ull);
      }
      moved = min(m, moved + __popc(mask));
    }
  }
}

// feeder: the host's tiles into the per-curve device rings (one warp, 32
// tiles a round)
__device__ __forceinline__ void serve_feeder(const ServeArgs& a) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t below = (1u << lane) - 1u;
  const uint64_t t0 = globaltimer_ns();
  uint64_t last = t0;
  uint64_t fed = a.dev->fed;
  uint64_t tail[3] = {a.dev->ring_tail[0], a.dev->ring_tail[1], a.dev->ring_tail[2]};
  uint64_t balanced = 0;
  uint32_t backoff = 64;
#pragma unroll 1
  for (uint32_t it = 0; it < SERVE_FEED_MAX_ITERS; ++it) {
    // the warp decides together: lane 0's clock and reads
    const uint64_t now = __shfl_sync(0xffffffffu, globaltimer_ns(), 0);
    const uint32_t stop = __shfl_sync(0xffffffffu, ld_acquire_sys_u32(&a.ctl->stop), 0);
    if (stop || now - last > a.idle_ns || now - t0 > a.life_ns) break;
    if (now - balanced > SERVE_BALANCE_NS) {
      serve_balance(a, lane, tail);
      balanced = now;
    }
    const uint64_t avail = __shfl_sync(0xffffffffu, ld_acquire_sys_u64(&a.ctl->tile_tail), 0);
    if (fed >= avail) {
      __nanosleep(backoff);
      backoff = backoff < 1024 ? 2 * backoff : 1024;
      continue;
    }
    backoff = 64;
    last = now;
    const uint64_t upto = avail - fed > 32 * 64 ? fed + 32 * 64 : avail;  // at most 64 rounds before re-reading the clock
#pragma unroll 1
    for (uint64_t b = fed; b < upto; b += 32) {
      const uint64_t t = b + lane;
      const bool valid = t < upto;
      uint4 v = make_uint4(0, 0, 0, 0);
      uint32_t curve = 3;
      if (valid) {
        v = ld_sys_v4(&a.htiles[(uint32_t)(t % a.tile_cap)]);
        curve = min(v.x >> 24, 2u);
      }
#pragma unroll
      for (uint32_t k = 0; k < 3; ++k) {
        const uint32_t m = __ballot_sync(0xffffffffu, curve == k);
        if (curve == k) {
          const uint64_t pos = tail[k] + __popc(m & below);
          a.tiles[(size_t)k * a.tile_cap + (uint32_t)(pos % a.tile_cap)] = ServeTile{v.x, v.y, v.z, v.w};
        }
        tail[k] += __popc(m);
      }
    }
    __threadfence();  // every lane's tiles before their publication
    __syncwarp();
    fed = upto;
    if (lane == 0) {
      a.dev->fed = fed;
#pragma unroll
      for (int k = 0; k < 3; ++k) st_release_gpu_u64(&a.dev->ring_tail[k], tail[k]);
      st_release_sys_u64(&a.ctl->tiles_fed, fed);
    }
    __syncwarp();
  }
  if (lane == 0) st_release_gpu_u32(&a.dev->closing, 1u);
}

// claim the next tile of ring k if it has one (lane 0)
__device__ __forceinline__ bool serve_claim(const ServeArgs& a, uint32_t k, uint64_t& pos) {
  uint64_t head = *(volatile uint64_t*)&a.dev->ring_head[k];
  const uint64_t tail = ld_acquire_gpu_u64(&a.dev->ring_tail[k]);
#pragma unroll 1
  while (head < tail) {
    const uint64_t prev = atomicCAS((unsigned long long*)&a.dev->ring_head[k], head, head + 1);
    if (prev == head) {
      pos = head;
      return true;
    }
    head = prev;
  }
  return false;
}

__device__ __forceinline__ uint64_t ring_waiting(const ServeArgs& a, uint32_t k) {
  const uint64_t tail = ld_acquire_gpu_u64(&a.dev->ring_tail[k]);
  const uint64_t head = *(volatile uint64_t*)&a.dev->ring_head[k];
  return tail > head ? tail - head : 0;
}

// lane 0: a tile of this TPC's curve (1), closed and empty (2), or the poll
// budget spent (0).  A TPC whose curve has no tile waiting and whose warps
// all finished theirs moves to the curve with the most tiles waiting.  After
// the close any ring's tile is taken: every published tile is processed
// before the kernel exits.
__device__ __forceinline__ uint32_t serve_next(const ServeArgs& a, uint32_t sm, uint32_t& curve, uint64_t& pos) {
  uint32_t* busy = &a.dev->busy[sm];
  uint32_t backoff = 128;
#pragma unroll 1
  for (uint32_t p = 0; p < SERVE_WAIT_MAX_POLLS; ++p) {
    const uint32_t cur = min(*(volatile uint32_t*)&a.dev->mode[sm], 2u);
    const uint64_t waiting = ring_waiting(a, cur);
    // without a backlog a TPC holds at most warp_cap tiles, so that light load
    // spreads over more TPCs (fewer warps per SM run faster) instead of
    // filling the TPCs already on the curve
    if (waiting && (waiting >= a.warp_cap || *(volatile uint32_t*)busy < a.warp_cap)) {
      atomicAdd(busy, 1u);  // counted from the claim on: the feeder sees the TPC's running tiles
      if (serve_claim(a, cur, pos)) {
        curve = cur;
        return 1;
      }
      atomicSub(busy, 1u);
      continue;
    }
    if (*(volatile uint32_t*)busy == 0) {
      // the TPC has no tile of its curve left: it moves to the curve with the most tiles waiting
      uint32_t best = cur;
      uint64_t most = 0;
#pragma unroll 1
      for (uint32_t j = 1; j < 3; ++j) {
        const uint32_t k = (cur + j) % 3;
        const uint64_t wt = ring_waiting(a, k);
        if (wt > most) {
          most = wt;
          best = k;
        }
      }
      if (best != cur) {
        if (atomicCAS(&a.dev->mode[sm], cur, best) == cur) atomicAdd(&a.dev->drains, 1ull);
        continue;
      }
    }
    if (ld_acquire_gpu_u32(&a.dev->closing)) {
      // the final tails are published before closing
#pragma unroll 1
      for (uint32_t k = 0; k < 3; ++k) {
        atomicAdd(busy, 1u);
        if (serve_claim(a, k, pos)) {
          curve = k;
          return 1;
        }
        atomicSub(busy, 1u);
      }
      return 2;
    }
    __nanosleep(backoff);
    backoff = backoff < 2048 ? 2 * backoff : 2048;
  }
  return 0;
}

// consumer warps: one tile at a time until the feeder closes and the rings are empty
constexpr int SERVE_MAX_SEGS = 4;  // tiles a warp works on at once (their items fill its 32 lanes)

// lane 0, after claiming the tile at `pos`: claim the next tiles of the same
// curve while their items still fit the warp's lanes (a request's last tile
// is mostly partial: a tenth of the lanes would idle).  Returns the tiles
// held; their positions in segs[].
__device__ __forceinline__ uint32_t serve_fill(const ServeArgs& a, uint32_t curve, uint64_t pos, uint64_t* segs) {
  const ServeTile* ring = a.tiles + (size_t)curve * a.tile_cap;
  segs[0] = pos;
  uint32_t cnt = 1, total = min((ring[(uint32_t)(pos % a.tile_cap)].shape >> 16) & 0xffu, 32u);
#pragma unroll 1
  while (cnt < SERVE_MAX_SEGS && total < 32) {
    const uint64_t tail = ld_acquire_gpu_u64(&a.dev->ring_tail[curve]);
    const uint64_t head = *(volatile uint64_t*)&a.dev->ring_head[curve];
    if (head >= tail) break;
    const uint32_t n = min((ring[(uint32_t)(head % a.tile_cap)].shape >> 16) & 0xffu, 32u);
    if (total + n > 32) break;
    if (atomicCAS((unsigned long long*)&a.dev->ring_head[curve], head, head + 1) != head) continue;  // taken meanwhile: look again
    segs[cnt++] = head;
    total += n;
  }
  return cnt;
}

// consumer warps: one group of tiles at a time until the feeder closes and the rings are empty
__device__ __forceinline__ void serve_consumer(const ServeArgs& a, uint32_t* stage) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t sm = (smid() / SERVE_SMS_PER_SLOT) % SERVE_MODE_SLOTS;
  if (lane == 0) *(volatile uint32_t*)&a.dev->seen[sm] = 1u;
#pragma unroll 1
  for (;;) {
    uint32_t got = 0, curve = 0, cnt = 0;
    uint64_t pos = 0, t_look = 0, t_got = 0;
    uint64_t segs[SERVE_MAX_SEGS] = {0, 0, 0, 0};
    if (lane == 0) {
      t_look = globaltimer_ns();
      got = serve_next(a, sm, curve, pos);
      if (got == 1) cnt = serve_fill(a, curve, pos, segs);
      t_got = globaltimer_ns();
      atomicAdd(&a.dev->idle_ns, (unsigned long long)(t_got - t_look));
      if (!got) atomicOr(&a.ctl->err, DEV_ERR_QUEUE_TIMEOUT);  // no tile and no close within the poll budget
    }
    got = __shfl_sync(0xffffffffu, got, 0);
    if (got != 1) return;
    curve = __shfl_sync(0xffffffffu, curve, 0);
    cnt = __shfl_sync(0xffffffffu, cnt, 0);
    // the tiles held: lanes base[j] .. base[j] + n[j] - 1 work on tile j
    ServeTile tl[SERVE_MAX_SEGS];
    uint32_t base[SERVE_MAX_SEGS], nseg[SERVE_MAX_SEGS];
    uint32_t total = 0;
#pragma unroll
    for (int j = 0; j < SERVE_MAX_SEGS; ++j) {
      const uint64_t p = __shfl_sync(0xffffffffu, segs[j], 0);
      tl[j] = ServeTile{0, 0, 0, 0};
      nseg[j] = 0;
      base[j] = total;
      if ((uint32_t)j < cnt) {
        tl[j] = a.tiles[(size_t)curve * a.tile_cap + (uint32_t)(p % a.tile_cap)];
        nseg[j] = min((tl[j].shape >> 16) & 0xffu, 32u - total);
        total += nseg[j];
      }
    }
    {  // inputs into the staging area: item base[j] + i of tile j at slot base[j] + i
      uint4* st4 = reinterpret_cast<uint4*>(stage);
#pragma unroll
      for (int j = 0; j < SERVE_MAX_SEGS; ++j) {
        const uint32_t n = nseg[j];
        uint4* dst = st4 + base[j] * 8;
        const uint8_t* sig = a.sig + (size_t)tl[j].first * 64;
        const uint8_t* msg = a.msg + (size_t)tl[j].first * 32;
        const uint8_t* pk = a.pk + (size_t)tl[j].first * 32;
#pragma unroll 1
        for (uint32_t c = lane; c < 4 * n; c += 32) dst[(c >> 2) * 8 + (c & 3)] = ld_sys_v4(sig + 16 * c);
#pragma unroll 1
        for (uint32_t c = lane; c < 2 * n; c += 32) dst[(c >> 1) * 8 + 4 + (c & 1)] = ld_sys_v4(msg + 16 * c);
        if (curve == 2) {
#pragma unroll 1
          for (uint32_t c = lane; c < 2 * n; c += 32) dst[(c >> 1) * 8 + 6 + (c & 1)] = ld_sys_v4(pk + 16 * c);
        }
      }
    }
    __syncwarp();
    uint32_t st = 0;
    if (lane < total) {
      uint32_t* w = stage + lane * 32;
      uint32_t o[16];
      if (curve == 0) st = serve_item<0>(w, w + 16, w + 24, a.tabs.k1, o);
      else if (curve == 1) st = serve_item<1>(w, w + 16, w + 24, a.tabs.r1, o);
      else st = serve_item<2>(w, w + 16, w + 24, a.tabs.ed, o);
#pragma unroll
      for (int k = 0; k < 16; ++k) w[k] = o[k];
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < SERVE_MAX_SEGS; ++j) {  // result records into the pinned output ring
      const uint32_t n = nseg[j];
      const uint4* src = reinterpret_cast<const uint4*>(stage) + base[j] * 8;
      uint4* out = reinterpret_cast<uint4*>(a.out + (size_t)tl[j].first * 64);
#pragma unroll 1
      for (uint32_t c = lane; c < 4 * n; c += 32) out[c] = src[(c >> 2) * 8 + (c & 3)];
      if (lane >= base[j] && lane < base[j] + n) a.st[tl[j].first + (lane - base[j])] = (uint8_t)st;
    }
    __threadfence_system();  // this lane's stores before the requests' completion entries
    __syncwarp();
    if (lane == 0) {
#pragma unroll
      for (int j = 0; j < SERVE_MAX_SEGS; ++j) {
        if ((uint32_t)j >= cnt) break;
        const uint32_t req = tl[j].shape & 0xffffu;
        if (atomicAdd(&a.count[req], nseg[j]) + nseg[j] == tl[j].target) {
          __threadfence_system();
          const uint64_t cpos = atomicAdd((unsigned long long*)&a.dev->comp_tail, 1ull);
          st_release_sys_u64(&a.comp[cpos % a.R], serve_completion(cpos, req, tl[j].seq));
        }
      }
      atomicSub(&a.dev->busy[sm], 1u);
      atomicAdd(&a.dev->tiles_done, (unsigned long long)cnt);
      atomicAdd(&a.dev->items_done, (unsigned long long)total);
      atomicAdd(&a.dev->work_ns, (unsigned long long)(globaltimer_ns() - t_got));
    }
  }
}

template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) serve_kernel(ServeArgs a) {
  __shared__ __align__(16) uint32_t stage_all[BLOCK / 32][SERVE_STAGE_WORDS];
  if (blockIdx.x == 0 && threadIdx.x < 32) serve_feeder(a);
  else serve_consumer(a, stage_all[threadIdx.x >> 5]);
  // the last warp out tells the host, which then needs no driver call to see the exit
  if ((threadIdx.x & 31u) == 0) {
    __threadfence_system();
    if (atomicSub(&a.dev->live_warps, 1u) == 1u) {
      __threadfence_system();
      st_release_sys_u32(&a.ctl->exited, a.launch);
    }
  }
}

// before each launch: the queue is open; TPCs start spread over the curves
__global__ void serve_reset_kernel(ServeDev* d, uint32_t warps) {
  d->closing = 0;
  d->live_warps = warps;
  for (int i = threadIdx.x; i < SERVE_MODE_SLOTS; i += blockDim.x) {
    d->mode[i] = i % 3;
    d->busy[i] = 0;
  }
}

}  // namespace sg
