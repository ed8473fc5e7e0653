// Kernel-side helpers shared by the plain and batched kernels.
#pragma once
#include <cuda_runtime.h>
#include "launch.h"
#include "tables.cuh"

namespace sg {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Wait for phase 0 of the mbarrier at shared address `bar`, at most max_polls
// polls (each try_wait also suspends in hardware for a bounded time); false
// when it did not complete.  Any device-side wait goes through here, so none
// can spin forever; the caller sets DEV_ERR_WAIT_TIMEOUT and returns.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t max_polls) {
  uint32_t done = 0;
  for (uint32_t i = 0; i < max_polls && !done; ++i) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar)
        : "memory");
  }
  return done != 0;
}

// Upper bound on mbarrier polls of a block waiting for its bulk copy (each
// try_wait also suspends in hardware for a bounded time: well under a second)
constexpr uint32_t STAGE_MAX_POLLS = 1u << 20;

// Copy `bytes` (a multiple of 16; both addresses 16-byte aligned) from global
// to shared memory with one bulk copy (TMA, non-multicast, this GPU's own
// memory) completing on an mbarrier; every thread of the block waits with a
// bounded poll.  When the wait runs out the block sets DEV_ERR_WAIT_TIMEOUT,
// waits once more (bounded) for its copy still in flight, and the caller
// returns.
__device__ __forceinline__ bool stage_to_smem(void* dst, const void* src, uint32_t bytes, uint64_t* bar, uint32_t* err) {
  const uint32_t b = smem_addr(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)), "l"(src),
                 "r"(bytes), "r"(b)
                 : "memory");
  }
  if (mbar_wait_bounded(b, STAGE_MAX_POLLS)) return true;
  if (threadIdx.x == 0) atomicOr(err, DEV_ERR_WAIT_TIMEOUT);
  (void)mbar_wait_bounded(b, STAGE_MAX_POLLS);
  return false;
}

__device__ __forceinline__ void load_words(const uint8_t* base, size_t idx, int nwords, uint32_t* w) {
  const uint4* p = reinterpret_cast<const uint4*>(base) + idx * (size_t)(nwords / 4);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if (q < nwords / 4) {
      uint4 v = __ldg(p + q);
      w[4 * q] = v.x; w[4 * q + 1] = v.y; w[4 * q + 2] = v.z; w[4 * q + 3] = v.w;
    }
  }
}

__device__ __forceinline__ void store_words(uint8_t* base, size_t idx, int nwords, const uint32_t* w) {
  uint4* p = reinterpret_cast<uint4*>(base) + idx * (size_t)(nwords / 4);
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (q < nwords / 4) p[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
}

}  // namespace sg
