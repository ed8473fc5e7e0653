// Modular inverse by Bernstein-Yang divsteps ("Fast constant-time gcd
// computation and modular inversion", 2019), batched 30 divsteps at a time on
// the low word, with the 2x2 transition matrix applied to the full-precision
// values in signed 30-bit limbs.  Replaces Fermat exponentiation (255
// squarings + ~15-60 multiplications) for the inverses on the hot path:
// r^-1 mod n and the projective-to-affine Z^-1 mod p.  (The reference uses a
// binary extended Euclid with a data-dependent loop, src/wgsl/ff.wgsl:60-120,
// which never terminates for 0.)
//
// The steps are the "half-delta" divsteps (delta starts at 1/2 instead of 1;
// the update rules are unchanged), for which 590 steps suffice for inputs
// below 2^256 (P. Wuille's safegcd bound analysis, as used by libsecp256k1's
// constant-time modular inverse); the original divsteps need 741 (the paper's
// floor((49 d + 57) / 17) for d = 256).  The iteration count is fixed at 20
// batches of 30 = 600 steps, so every lane of a warp runs the same
// instruction stream.  delta is kept doubled (2 delta, odd) in an int32.
// Callers check x * inv == 1 and fall back to Fermat, which only a broken
// bound could trigger.
#pragma once
#include "arith.cuh"

namespace sg {

constexpr int DIVSTEP_BATCHES = 20;  // of 30 half-delta divsteps

struct S30 {  // value = sum v[i] 2^(30 i); v[0..7] in [0, 2^30), v[8] signed
  int32_t v[9];
};

constexpr int32_t M30 = 0x3fffffff;

SG_HD S30 s30_from_u256(const u256& x) {
  S30 s;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const int bit = 30 * i, w = bit >> 5, sh = bit & 31;
    uint64_t lo = x.w[w];
    uint64_t hi = (w + 1 < 8) ? x.w[w + 1] : 0;
    uint64_t cat = lo | (hi << 32);
    s.v[i] = (int32_t)((cat >> sh) & (i < 8 ? (uint64_t)M30 : 0xffffffffull));
  }
  return s;
}

// 30 divsteps on the low 32 bits of f and g (two's complement).  delta2 is
// 2 delta; returns the new value; t = (u, v, q, r) with u f + v g = f' 2^30,
// q f + r g = g' 2^30.
SG_HD int32_t divsteps30(int32_t delta2, uint32_t f, uint32_t g, int32_t t[4]) {
  int32_t u = 1, v = 0, q = 0, r = 1;
#pragma unroll
  for (int i = 0; i < 30; ++i) {
    const bool odd = (g & 1u) != 0;
    const bool sw = odd && delta2 > 0;
    // swap case: (f, g) <- (g, -f), (u, v, q, r) <- (q, r, -u, -v), delta <- -delta
    const uint32_t f1 = sw ? g : f;
    const uint32_t g1 = sw ? (0u - f) : g;
    const int32_t u1 = sw ? q : u, v1 = sw ? r : v;
    const int32_t q1 = sw ? -u : q, r1 = sw ? -v : r;
    delta2 = sw ? -delta2 : delta2;
    // odd g: g += f, (q, r) += (u, v)
    const uint32_t g2 = odd ? g1 + f1 : g1;
    const int32_t q2 = odd ? q1 + u1 : q1, r2 = odd ? r1 + v1 : r1;
    f = f1;
    g = g2 >> 1;
    u = u1 * 2;
    v = v1 * 2;
    q = q2;
    r = r2;
    delta2 += 2;  // delta += 1
  }
  t[0] = u;
  t[1] = v;
  t[2] = q;
  t[3] = r;
  return delta2;
}

// (f, g) <- (u f + v g, q f + r g) / 2^30, exact
SG_HD void s30_update_fg(S30& f, S30& g, const int32_t t[4]) {
  SG_COUNT_MULS(2 * 4 * 9);  // 36 wide products
  const int64_t u = t[0], v = t[1], q = t[2], r = t[3];
  int64_t cf = u * f.v[0] + v * g.v[0];
  int64_t cg = q * f.v[0] + r * g.v[0];
  cf >>= 30;
  cg >>= 30;
#pragma unroll
  for (int i = 1; i < 9; ++i) {
    cf += u * f.v[i] + v * g.v[i];
    cg += q * f.v[i] + r * g.v[i];
    f.v[i - 1] = (int32_t)(cf & M30);
    g.v[i - 1] = (int32_t)(cg & M30);
    cf >>= 30;
    cg >>= 30;
  }
  f.v[8] = (int32_t)cf;
  g.v[8] = (int32_t)cg;
}

// (d, e) <- (u d + v e, q d + r e) / 2^30 mod M, keeping both in (-2M, M):
// a multiple of M chosen to clear the low 30 bits is added before the shift
SG_HD void s30_update_de(S30& d, S30& e, const int32_t t[4], const S30& M, uint32_t minv30) {
  SG_COUNT_MULS(2 * 6 * 9 + 2);  // 54 wide products and two low ones
  const int32_t u = t[0], v = t[1], q = t[2], r = t[3];
  const int32_t sd = d.v[8] >> 31, se = e.v[8] >> 31;
  int32_t md = (u & sd) + (v & se);
  int32_t me = (q & sd) + (r & se);
  int64_t cd = (int64_t)u * d.v[0] + (int64_t)v * e.v[0];
  int64_t ce = (int64_t)q * d.v[0] + (int64_t)r * e.v[0];
  md -= (int32_t)((minv30 * (uint32_t)cd + (uint32_t)md) & (uint32_t)M30);
  me -= (int32_t)((minv30 * (uint32_t)ce + (uint32_t)me) & (uint32_t)M30);
  cd += (int64_t)M.v[0] * md;
  ce += (int64_t)M.v[0] * me;
  cd >>= 30;
  ce >>= 30;
#pragma unroll
  for (int i = 1; i < 9; ++i) {
    cd += (int64_t)u * d.v[i] + (int64_t)v * e.v[i] + (int64_t)M.v[i] * md;
    ce += (int64_t)q * d.v[i] + (int64_t)r * e.v[i] + (int64_t)M.v[i] * me;
    d.v[i - 1] = (int32_t)(cd & M30);
    e.v[i - 1] = (int32_t)(ce & M30);
    cd >>= 30;
    ce >>= 30;
  }
  d.v[8] = (int32_t)cd;
  e.v[8] = (int32_t)ce;
}

// signed value of s as a 256-bit word vector plus a signed top word
SG_HD void s30_to_wide(const S30& s, u256& lo, int32_t& top) {
  u256 x = u256_zero();
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int bit = 30 * i, w = bit >> 5, sh = bit & 31;
    const uint64_t val = (uint64_t)(uint32_t)s.v[i] << sh;
    x.w[w] |= (uint32_t)val;
    if (w + 1 < 8) x.w[w + 1] |= (uint32_t)(val >> 32);
  }
  // + v[8] * 2^240 (bit 16 of word 7)
  const int64_t t7 = (int64_t)x.w[7] + ((int64_t)s.v[8] << 16);
  x.w[7] = (uint32_t)t7;
  top = (int32_t)(t7 >> 32);
  lo = x;
}

// x^-1 mod M for 0 < x < M, M odd, gcd(x, M) = 1 (returns 0 for x = 0).
// A called function: the modulus is an argument, so every field of a kernel
// (p and n of each curve) shares one copy of the divstep code, which keeps
// the code that out-of-phase warps need at once small.
SG_NOINL u256 divstep_inverse(const u256& x, const u256& Mu, uint32_t minv30) {
  const S30 M = s30_from_u256(Mu);
  S30 f = M, g = s30_from_u256(x), d, e;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    d.v[i] = 0;
    e.v[i] = 0;
  }
  e.v[0] = 1;
  int32_t delta2 = 1;  // delta = 1/2
#pragma unroll 1
  for (int it = 0; it < DIVSTEP_BATCHES; ++it) {
    int32_t t[4];
    delta2 = divsteps30(delta2, (uint32_t)f.v[0] | ((uint32_t)f.v[1] << 30), (uint32_t)g.v[0] | ((uint32_t)g.v[1] << 30), t);
    s30_update_de(d, e, t, M, minv30);
    s30_update_fg(f, g, t);
#ifdef __CUDA_ARCH__
    // once g = 0 further batches only keep f = +-1 and change d by multiples
    // of M, so the warp stops when all of its lanes are there (random inputs
    // get there after 17 or 18 batches).  The host build runs every batch, so
    // the multiply counts taken from it stay an upper bound.
    if (it >= 12) {
      uint32_t nz = 0;
#pragma unroll
      for (int k = 0; k < 9; ++k) nz |= (uint32_t)g.v[k];
      if (__all_sync(__activemask(), nz == 0)) break;
    }
#endif
  }
  // now g = 0 and f = +-1: x^-1 = sign(f) * d, with d in (-2M, M)
  u256 lo;
  int32_t top;
  s30_to_wide(d, lo, top);
  if (f.v[8] < 0) {  // negate (two's complement over 256 + 32 bits)
    u256 z = u256_zero(), nl;
    uint32_t bw = u256_sub(nl, z, lo);
    lo = nl;
    top = -top - (int32_t)bw;
  }
  // range (-2M, 2M): add M while negative (twice at most), then subtract M once if >= M
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (top < 0) {
      u256 s;
      uint32_t c = u256_add(s, lo, Mu);
      lo = s;
      top += (int32_t)c;
    }
  }
  if (top > 0 || u256_gte(lo, Mu)) {
    u256 s;
    u256_sub(s, lo, Mu);
    lo = s;
  }
  return lo;
}

}  // namespace sg
