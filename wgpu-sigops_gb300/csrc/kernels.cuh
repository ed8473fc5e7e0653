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
