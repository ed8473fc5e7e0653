// Plain kernels: one signature per thread, one curve per launch.
//
// They replace the reference's one-kernel entry points secp256k1_recover_main /
// secp256r1_recover_main / ed25519_verify_main
// (src/wgsl/main/secp256k1_ecdsa_main.wgsl:22-82 and siblings) and their
// multi-stage variants (src/wgsl/main/*_main_{0..5}.wgsl), which split the same
// work into 5-6 dispatches with intermediates in global memory.  Each thread
// handles one signature; generator-table entries are read from global memory
// (L2-resident) as the windows need them.
#pragma once
#include <type_traits>

#include "kernels.cuh"
#include "launch.h"

namespace sg {

// One item per thread; the grid covers the batch.  With no loop state live across the arithmetic the
// 128 x 3 shape (at most 170 registers, 12 warps per SM) runs without spills.
template <class T, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) ecdsa_plain_kernel(const uint8_t* __restrict__ sigs, const uint8_t* __restrict__ msgs,
                                                             size_t n, const uint32_t* __restrict__ gtab, uint8_t* __restrict__ out,
                                                             uint8_t* __restrict__ status, uint32_t* err) {
  // secp256k1 recovers with the GLV split: its table holds the multiples of G
  // and of 2^128 G
  constexpr bool GLV = std::is_same<T, K1Traits>::value;
  const size_t i = (size_t)blockIdx.x * BLOCK + threadIdx.x;
  if (i >= n) return;
  uint32_t s[16], m[8], o[16];
  load_words(sigs, i, 16, s);
  load_words(msgs, i, 8, m);
  uint8_t st = ecdsa_recover<T, GLV>(s, m, gtab, o);
  store_words(out, i, 16, o);
  status[i] = st;
}

}  // namespace sg
