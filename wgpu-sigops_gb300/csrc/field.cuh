// Prime fields for the three curves, 8 x 32-bit limbs.  The scalar fields
// keep values canonical (in [0, p)) after every operation; the three base
// fields keep them below 2^256 only (weakly reduced) and make them canonical
// (canon) where a comparison or an encoding needs it.  The base-field multiply and square are
// called functions, not inlined: the hot loops then fit the instruction cache
// (inlining them everywhere measured 4% slower overall, 19% on ed25519, and
// took six times longer to compile).
//
//  * FpK1  p = 2^256 - 2^32 - 977   special-form fold (2^256 = 2^32 + 977)
//  * FpEd  p = 2^255 - 19           special-form fold (2^256 = 38)
//  * FpR1  p = NIST P-256           Montgomery form, multiply-free reduction rounds
//  * Mont<...> generic Montgomery (CIOS) for the scalar fields mod n and mod l
//
// The reference does all of this with 13-bit limbs: Barrett `ff_mul`
// (src/wgsl/ff.wgsl:122-198), CIOS `mont_mul` (src/wgsl/mont.wgsl:5-78),
// square-and-multiply `modpow` (src/wgsl/mont.wgsl:80-99), binary-EEA
// `ff_inverse` (src/wgsl/ff.wgsl:60-120) and the (p+1)/4 square root
// (src/wgsl/secp256k1_curve.wgsl:12-21).  Here exponentiations use fixed
// addition chains (253-255 squarings and 7-15 multiplications each) and the
// inverses use a fixed count of Bernstein-Yang divsteps (inverse.cuh), each
// verified by one multiplication with Fermat as the fallback, so no input can
// make a loop run away (the reference's binary EEA never terminates for 0).
#pragma once
#include "arith.cuh"
#include "inverse.cuh"

namespace sg {

#define SG_U256(a0, a1, a2, a3, a4, a5, a6, a7) \
  u256 { { a0, a1, a2, a3, a4, a5, a6, a7 } }

// ---------------------------------------------------------------------------
// shared helpers
// ---------------------------------------------------------------------------

// r = (a + b) mod m for a, b < m
SG_HD u256 mod_add(const u256& a, const u256& b, const u256& m) {
  u256 t, u;
  uint32_t c = u256_add(t, a, b);
  uint32_t bw = u256_sub(u, t, m);
  return u256_select(c | (bw ^ 1u), u, t);
}

// r = (a - b) mod m for a, b < m
SG_HD u256 mod_sub(const u256& a, const u256& b, const u256& m) {
  u256 t, u;
  uint32_t bw = u256_sub(t, a, b);
  u256_add(u, t, m);
  return u256_select(bw != 0, u, t);
}

SG_HD u256 mod_neg(const u256& a, const u256& m) {
  u256 t;
  u256_sub(t, m, a);
  return u256_select(u256_is_zero(a), a, t);
}

// reduce x < 2^256 into [0, m) when m > 2^255 (at most one subtraction)
SG_HD u256 reduce_once(const u256& x, const u256& m) {
  u256 t;
  uint32_t bw = u256_sub(t, x, m);
  return u256_select(bw == 0, t, x);
}

// ---------------------------------------------------------------------------
// secp256k1 base field
// ---------------------------------------------------------------------------
struct FpK1 {
  SG_HD static u256 P() { return SG_U256(0xfffffc2fu, 0xfffffffeu, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu); }

  // t = H * 2^256 + L  ==  L + H * 977 + H * 2^32  (mod p), weakly reduced
  // (below 2^256)
  SG_HD static u256 reduce(const uint32_t t[16]) {
    uint32_t v[10];
    // v = L + lo(H_j * 977) at column j
    v[0] = mad_lo_cc(t[8], 977u, t[0]);
#pragma unroll
    for (int j = 1; j < 8; ++j) v[j] = madc_lo_cc(t[8 + j], 977u, t[j]);
    v[8] = addc(0u, 0u);
    // + hi(H_j * 977) at column j+1
    v[1] = mad_hi_cc(t[8], 977u, v[1]);
#pragma unroll
    for (int j = 1; j < 7; ++j) v[j + 1] = madc_hi_cc(t[8 + j], 977u, v[j + 1]);
    v[8] = madc_hi(t[15], 977u, v[8]);  // < 2^32: hi(.) < 977 and v[8] <= 1
    // + H_j at column j+1
    v[1] = add_cc(v[1], t[8]);
#pragma unroll
    for (int j = 1; j < 8; ++j) v[j + 1] = addc_cc(v[j + 1], t[8 + j]);
    v[9] = addc(0u, 0u);
    // second fold of the top 33 bits, top = v[8] + v[9] 2^32 (v[9] <= 1), as
    // one three-word addend: top (2^32 + 977) = a0 + a1 2^32 + a2 2^64 with
    // a0 = lo(v8 977), a1 = hi(v8 977) + v8 + v9 977, a2 = v9 + carry
    const uint32_t s1 = mul_hi(v[8], 977u) + v[9] * 977u;  // < 2 * 977
    const uint32_t a0 = mul_lo(v[8], 977u);
    const uint32_t a1 = add_cc(v[8], s1);
    const uint32_t a2 = addc(v[9], 0u);
    u256 r;
    r.w[0] = add_cc(v[0], a0);
    r.w[1] = addc_cc(v[1], a1);
    r.w[2] = addc_cc(v[2], a2);
#pragma unroll
    for (int j = 3; j < 8; ++j) r.w[j] = addc_cc(v[j], 0u);
    const uint32_t c = addc(0u, 0u);
    // a carry out leaves r below 2^66: adding 2^32 + 977 back reaches word 2
    // at most
    r.w[0] = add_cc(r.w[0], c * 977u);
    r.w[1] = addc_cc(r.w[1], c);
    r.w[2] = addc(r.w[2], 0u);
    return r;
  }

  SG_HD static u256 canon(const u256& x) { return reduce_once(x, P()); }  // x < 2^256 < 2p
  SG_HD static bool is_zero(const u256& a) { return u256_is_zero(a) || u256_eq(a, P()); }  // a == 0 mod p
  SG_NOINL static u256 mul(const u256 a, const u256 b) { uint32_t t[16]; mul_wide(t, a, b); return reduce(t); }
  SG_NOINL static u256 sqr(const u256 a) { uint32_t t[16]; sqr_wide(t, a); return reduce(t); }
  // a + b for a, b < 2^256, weakly reduced: a carry out of 2^256 is worth
  // 2^32 + 977.  Adding it back carries again only when the sum left words
  // 2..7 zero and word 1 at most 1, so the second correction touches words 0
  // and 1 alone.
  SG_HD static u256 add(const u256& a, const u256& b) {
    u256 t;
    const uint32_t c = u256_add(t, a, b);
    t.w[0] = add_cc(t.w[0], c * 977u);
    t.w[1] = addc_cc(t.w[1], c);
#pragma unroll
    for (int j = 2; j < 8; ++j) t.w[j] = addc_cc(t.w[j], 0u);
    const uint32_t c2 = addc(0u, 0u);
    t.w[0] = add_cc(t.w[0], c2 * 977u);
    t.w[1] = addc(t.w[1], c2);
    return t;
  }
  // a - b for a, b < 2^256, weakly reduced: a borrow is worth -(2^32 + 977);
  // a second borrow leaves words 2..7 all ones and word 1 at least 2^32 - 2,
  // so its correction touches words 0 and 1 alone
  SG_HD static u256 sub(const u256& a, const u256& b) {
    u256 t;
    const uint32_t bw = u256_sub(t, a, b);
    t.w[0] = sub_cc(t.w[0], bw * 977u);
    t.w[1] = subc_cc(t.w[1], bw);
#pragma unroll
    for (int j = 2; j < 8; ++j) t.w[j] = subc_cc(t.w[j], 0u);
    const uint32_t bw2 = subc(0u, 0u) & 1u;
    t.w[0] = sub_cc(t.w[0], bw2 * 977u);
    t.w[1] = subc(t.w[1], bw2);
    return t;
  }
  // a / 2 mod p for a < 2^256, weakly reduced: (a + p) / 2 when a is odd
  SG_HD static u256 half(const u256& a) {
    const uint32_t m = 0u - (a.w[0] & 1u);
    const u256 p = P();
    u256 t;
    t.w[0] = add_cc(a.w[0], p.w[0] & m);
#pragma unroll
    for (int j = 1; j < 8; ++j) t.w[j] = addc_cc(a.w[j], p.w[j] & m);
    const uint32_t c = addc(0u, 0u);
    u256 r;
#pragma unroll
    for (int j = 0; j < 7; ++j) r.w[j] = (t.w[j] >> 1) | (t.w[j + 1] << 31);
    r.w[7] = (t.w[7] >> 1) | (c << 31);
    return r;
  }
  SG_HD static u256 neg(const u256& a) { return sub(u256_zero(), a); }  // 0 - 0 = 0 without a borrow
  SG_HD static u256 one() { return u256_small(1); }
  SG_HD static u256 zero() { return u256_zero(); }
  SG_HD static u256 from_int(const u256& x) { return canon(x); }  // x < 2^256
  SG_HD static u256 to_int(const u256& a) { return canon(a); }
  SG_HD static u256 sqr_n(u256 a, int n) {
#pragma unroll 1
    for (int i = 0; i < n; ++i) a = sqr(a);
    return a;
  }

  // x2 .. x223: a^(2^k - 1) blocks shared by the inverse and the square root
  SG_HD static void blocks(const u256 a, u256& x2, u256& x22, u256& x223) {
    x2 = mul(sqr(a), a);
    u256 x3 = mul(sqr(x2), a);
    u256 x6 = mul(sqr_n(x3, 3), x3);
    u256 x9 = mul(sqr_n(x6, 3), x3);
    u256 x11 = mul(sqr_n(x9, 2), x2);
    x22 = mul(sqr_n(x11, 11), x11);
    u256 x44 = mul(sqr_n(x22, 22), x22);
    u256 x88 = mul(sqr_n(x44, 44), x44);
    u256 x176 = mul(sqr_n(x88, 88), x88);
    u256 x220 = mul(sqr_n(x176, 44), x44);
    x223 = mul(sqr_n(x220, 3), x3);
  }

  // a^-1 by divsteps (canonical result), verified; Fermat fallback
  SG_NOINL static u256 inv(const u256 a) {
    const u256 ac = canon(a);
    u256 r = divstep_inverse(ac, P(), 0x2ddacacfu);
    return u256_eq(canon(mul(ac, r)), one()) ? r : canon(inv_fermat(ac));
  }

  // a^(p-2): 255 squarings, 15 multiplications
  SG_NOINL static u256 inv_fermat(const u256 a) {
    u256 x2, x22, t;
    blocks(a, x2, x22, t);
    t = mul(sqr_n(t, 23), x22);
    t = mul(sqr_n(t, 5), a);
    t = mul(sqr_n(t, 3), x2);
    t = mul(sqr_n(t, 2), a);
    return t;
  }

  // a^((p+1)/4): 253 squarings, 13 multiplications
  SG_NOINL static u256 sqrt_candidate(const u256 a) {
    u256 x2, x22, t;
    blocks(a, x2, x22, t);
    t = mul(sqr_n(t, 23), x22);
    t = mul(sqr_n(t, 6), x2);
    t = sqr_n(t, 2);
    return t;
  }
};

// ---------------------------------------------------------------------------
// ed25519 base field
// ---------------------------------------------------------------------------
struct FpEd {
  SG_HD static u256 P() { return SG_U256(0xffffffedu, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0x7fffffffu); }

  // x < 2^256  ->  x mod p  (2^255 = 19)
  SG_HD static u256 canon(u256 x) {
    uint32_t top = x.w[7] >> 31;
    x.w[7] &= 0x7fffffffu;
    x.w[0] = add_cc(x.w[0], top * 19u);
#pragma unroll
    for (int j = 1; j < 8; ++j) x.w[j] = addc_cc(x.w[j], 0u);
    // now x < 2^255 + 19; subtract p when x + 19 >= 2^255
    u256 y;
    y.w[0] = add_cc(x.w[0], 19u);
#pragma unroll
    for (int j = 1; j < 8; ++j) y.w[j] = addc_cc(x.w[j], 0u);
    bool ge = (y.w[7] >> 31) != 0;
    y.w[7] &= 0x7fffffffu;
    return u256_select(ge, y, x);
  }

  // t = H * 2^256 + L  ==  L + 38 H  (mod p), weakly reduced (below 2^256)
  SG_HD static u256 reduce(const uint32_t t[16]) {
    uint32_t v[9];
    v[0] = mad_lo_cc(t[8], 38u, t[0]);
#pragma unroll
    for (int j = 1; j < 8; ++j) v[j] = madc_lo_cc(t[8 + j], 38u, t[j]);
    v[8] = addc(0u, 0u);
    v[1] = mad_hi_cc(t[8], 38u, v[1]);
#pragma unroll
    for (int j = 1; j < 7; ++j) v[j + 1] = madc_hi_cc(t[8 + j], 38u, v[j + 1]);
    v[8] = madc_hi(t[15], 38u, v[8]);  // v[8] <= 38
    u256 r;
    r.w[0] = mad_lo_cc(v[8], 38u, v[0]);
#pragma unroll
    for (int j = 1; j < 8; ++j) r.w[j] = addc_cc(v[j], 0u);
    const uint32_t c = addc(0u, 0u);
    // a carry out leaves r below 38 * 38 + 38: adding 38 back stays in word 0
    r.w[0] += c * 38u;
    return r;
  }

  // the ed25519 kernel is bound by the wide/high multiply pipe: its products
  // use one Karatsuba level (96 multiplies instead of 128; measured +3% there,
  // while the latency-bound secp256k1 / P-256 kernels gain nothing from it)
  SG_NOINL static u256 mul(const u256 a, const u256 b) { uint32_t t[16]; mul_wide_kara(t, a, b); return reduce(t); }
  SG_NOINL static u256 sqr(const u256 a) { uint32_t t[16]; sqr_wide(t, a); return reduce(t); }
  // a + b for a, b < 2^256, weakly reduced: a carry out of 2^256 is worth 38.
  // Adding it back can carry once more only when the sum left t.w[0] < 38
  // and the other words zero, so the second correction touches word 0 alone.
  SG_HD static u256 add(const u256& a, const u256& b) {
    u256 t;
    const uint32_t c = u256_add(t, a, b);
    t.w[0] = add_cc(t.w[0], c * 38u);
#pragma unroll
    for (int j = 1; j < 8; ++j) t.w[j] = addc_cc(t.w[j], 0u);
    const uint32_t c2 = addc(0u, 0u);
    t.w[0] += c2 * 38u;
    return t;
  }
  // a - b for a, b < 2^256, weakly reduced: a borrow is worth -38; a second
  // borrow leaves t.w[0] >= 2^32 - 38, so its correction touches word 0 alone
  SG_HD static u256 sub(const u256& a, const u256& b) {
    u256 t;
    const uint32_t bw = u256_sub(t, a, b);
    t.w[0] = sub_cc(t.w[0], bw * 38u);
#pragma unroll
    for (int j = 1; j < 8; ++j) t.w[j] = subc_cc(t.w[j], 0u);
    const uint32_t bw2 = subc(0u, 0u) & 1u;
    t.w[0] -= bw2 * 38u;
    return t;
  }
  SG_HD static u256 neg(const u256& a) { return sub(u256_zero(), a); }  // 0 - 0 = 0 without a borrow
  SG_HD static u256 one() { return u256_small(1); }
  SG_HD static u256 zero() { return u256_zero(); }
  SG_HD static u256 from_int(const u256& x) { return canon(x); }
  SG_HD static u256 to_int(const u256& a) { return canon(a); }
  SG_HD static u256 D() { return SG_U256(0x135978a3u, 0x75eb4dcau, 0x4141d8abu, 0x00700a4du, 0x7779e898u, 0x8cc74079u, 0x2b6ffe73u, 0x52036ceeu); }
  SG_HD static u256 D2() { return SG_U256(0x26b2f159u, 0xebd69b94u, 0x8283b156u, 0x00e0149au, 0xeef3d130u, 0x198e80f2u, 0x56dffce7u, 0x2406d9dcu); }
  SG_HD static u256 SQRT_M1() { return SG_U256(0x4a0ea0b0u, 0xc4ee1b27u, 0xad2fe478u, 0x2f431806u, 0x3dfbd7a7u, 0x2b4d0099u, 0x4fc1df0bu, 0x2b832480u); }

  SG_HD static u256 sqr_n(u256 a, int n) {
#pragma unroll 1
    for (int i = 0; i < n; ++i) a = sqr(a);
    return a;
  }

  // z^(2^250 - 1) and z^11 (the shared prefix of the inverse and the p58 power)
  SG_HD static void pow250(const u256 z, u256& z2_250_0, u256& z11) {
    u256 z2 = sqr(z);
    u256 z9 = mul(sqr_n(z2, 2), z);
    z11 = mul(z9, z2);
    u256 z2_5_0 = mul(sqr(z11), z9);
    u256 z2_10_0 = mul(sqr_n(z2_5_0, 5), z2_5_0);
    u256 z2_20_0 = mul(sqr_n(z2_10_0, 10), z2_10_0);
    u256 z2_40_0 = mul(sqr_n(z2_20_0, 20), z2_20_0);
    u256 z2_50_0 = mul(sqr_n(z2_40_0, 10), z2_10_0);
    u256 z2_100_0 = mul(sqr_n(z2_50_0, 50), z2_50_0);
    u256 z2_200_0 = mul(sqr_n(z2_100_0, 100), z2_100_0);
    z2_250_0 = mul(sqr_n(z2_200_0, 50), z2_50_0);
  }

  // z^-1 by divsteps (canonical result), verified; Fermat fallback
  SG_NOINL static u256 inv(const u256 z) {
    const u256 zc = canon(z);
    u256 r = divstep_inverse(zc, P(), 0x179435e5u);
    return u256_eq(canon(mul(zc, r)), one()) ? r : canon(inv_fermat(zc));
  }

  // z^(p-2) = z^(2^255 - 21)
  SG_NOINL static u256 inv_fermat(const u256 z) {
    u256 t, z11;
    pow250(z, t, z11);
    return mul(sqr_n(t, 5), z11);
  }

  // z^((p-5)/8) = z^(2^252 - 3)
  SG_NOINL static u256 pow_p58(const u256 z) {
    u256 t, z11;
    pow250(z, t, z11);
    return mul(sqr_n(t, 2), z);
  }
};

// ---------------------------------------------------------------------------
// Generic Montgomery arithmetic, R = 2^256 (CIOS with even/odd carry chains)
// ---------------------------------------------------------------------------
// Row i adds a * b_i and then m * N (m = t0 * n0'), each as an even-limb and
// an odd-limb carry chain, and drops the (now zero) low word.  Inlined: as a
// called function (one copy for every scalar field) secp256k1 signatures took
// 3-4% longer.
SG_HD u256 mont_mul(const u256& a, const u256& b, const u256& N, uint32_t ninv) {
  uint32_t t[10];
#pragma unroll
  for (int k = 0; k < 10; ++k) t[k] = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint32_t bi = b.w[i];
    t[0] = mad_lo_cc(a.w[0], bi, t[0]);
    t[1] = madc_hi_cc(a.w[0], bi, t[1]);
#pragma unroll
    for (int j = 2; j < 8; j += 2) {
      t[j] = madc_lo_cc(a.w[j], bi, t[j]);
      t[j + 1] = madc_hi_cc(a.w[j], bi, t[j + 1]);
    }
    t[8] = addc_cc(t[8], 0u);
    t[9] = addc(t[9], 0u);
    t[1] = mad_lo_cc(a.w[1], bi, t[1]);
    t[2] = madc_hi_cc(a.w[1], bi, t[2]);
#pragma unroll
    for (int j = 3; j < 8; j += 2) {
      t[j] = madc_lo_cc(a.w[j], bi, t[j]);
      t[j + 1] = madc_hi_cc(a.w[j], bi, t[j + 1]);
    }
    t[9] = addc(t[9], 0u);

    const uint32_t m = mul_lo(t[0], ninv);
    t[0] = mad_lo_cc(m, N.w[0], t[0]);
    t[1] = madc_hi_cc(m, N.w[0], t[1]);
#pragma unroll
    for (int j = 2; j < 8; j += 2) {
      t[j] = madc_lo_cc(m, N.w[j], t[j]);
      t[j + 1] = madc_hi_cc(m, N.w[j], t[j + 1]);
    }
    t[8] = addc_cc(t[8], 0u);
    t[9] = addc(t[9], 0u);
    t[1] = mad_lo_cc(m, N.w[1], t[1]);
    t[2] = madc_hi_cc(m, N.w[1], t[2]);
#pragma unroll
    for (int j = 3; j < 8; j += 2) {
      t[j] = madc_lo_cc(m, N.w[j], t[j]);
      t[j + 1] = madc_hi_cc(m, N.w[j], t[j + 1]);
    }
    t[9] = addc(t[9], 0u);
    // shift down one word
#pragma unroll
    for (int k = 0; k < 9; ++k) t[k] = t[k + 1];
    t[9] = 0;
  }
  // t < 2N: subtract N once when t >= N
  u256 r, s;
#pragma unroll
  for (int k = 0; k < 8; ++k) r.w[k] = t[k];
  uint32_t bw = u256_sub(s, r, N);
  return u256_select((t[8] != 0) | (bw == 0), s, r);
}

template <class C>
struct Mont {
  SG_HD static u256 N() { return C::N(); }
  SG_HD static u256 mul(const u256& a, const u256& b) { return mont_mul(a, b, C::N(), C::NINV); }
  SG_HD static u256 sqr(const u256& a) { return mont_mul(a, a, C::N(), C::NINV); }
  SG_HD static u256 add(const u256& a, const u256& b) { return mod_add(a, b, C::N()); }
  SG_HD static u256 sub(const u256& a, const u256& b) { return mod_sub(a, b, C::N()); }
  SG_HD static u256 neg(const u256& a) { return mod_neg(a, C::N()); }
  SG_HD static u256 zero() { return u256_zero(); }
  SG_HD static u256 one() { return C::ONE_MONT(); }                 // R mod N
  SG_HD static u256 from_int(const u256& x) { return mul(x, C::R2()); }  // any x < 2^256
  SG_HD static u256 to_int(const u256& a) { return mul(a, u256_small(1)); }
  SG_HD static u256 sqr_n(u256 a, int n) {
#pragma unroll 1
    for (int i = 0; i < n; ++i) a = sqr(a);
    return a;
  }
  // a^e for a constant exponent given as 8 little-endian words, 4-bit window
  SG_HD static u256 pow_const(const u256 a, const uint32_t* e) {
    u256 tab[16];
    tab[0] = one();
    tab[1] = a;
#pragma unroll 1
    for (int k = 2; k < 16; ++k) tab[k] = mul(tab[k - 1], a);
    u256 r = tab[e[7] >> 28];
#pragma unroll 1
    for (int i = 62; i >= 0; --i) {
      r = sqr_n(r, 4);
      uint32_t nib = (e[i >> 3] >> ((i & 7) * 4)) & 15u;
      if (nib) r = mul(r, tab[nib]);
    }
    return r;
  }
  // x^-1 for a plain integer 0 < x < N: divsteps, verified; Fermat fallback
  SG_NOINL static u256 inv_int(const u256 x) {
    u256 r = divstep_inverse(x, C::N(), C::MINV30);
    if (u256_eq(mul(from_int(x), r), u256_small(1))) return r;
    return to_int(inv(from_int(x)));
  }

  // Fermat inverse in the Montgomery domain
  SG_NOINL static u256 inv(const u256 a) {
    uint32_t e[8];
    u256 m2 = C::N_MINUS_2();
#pragma unroll
    for (int k = 0; k < 8; ++k) e[k] = m2.w[k];
    return pow_const(a, e);
  }
};

struct K1ScalarC {
  SG_HD static u256 N() { return SG_U256(0xd0364141u, 0xbfd25e8cu, 0xaf48a03bu, 0xbaaedce6u, 0xfffffffeu, 0xffffffffu, 0xffffffffu, 0xffffffffu); }
  SG_HD static u256 R2() { return SG_U256(0x67d7d140u, 0x896cf214u, 0x0e7cf878u, 0x741496c2u, 0x5bcd07c6u, 0xe697f5e4u, 0x81c69bc5u, 0x9d671cd5u); }
  SG_HD static u256 ONE_MONT() { return SG_U256(0x2fc9bebfu, 0x402da173u, 0x50b75fc4u, 0x45512319u, 0x00000001u, 0x00000000u, 0x00000000u, 0x00000000u); }
  SG_HD static u256 N_MINUS_2() { return SG_U256(0xd036413fu, 0xbfd25e8cu, 0xaf48a03bu, 0xbaaedce6u, 0xfffffffeu, 0xffffffffu, 0xffffffffu, 0xffffffffu); }
  static constexpr uint32_t NINV = 0x5588b13fu;
  static constexpr uint32_t MINV30 = 0x2a774ec1u;
};

struct R1ScalarC {
  SG_HD static u256 N() { return SG_U256(0xfc632551u, 0xf3b9cac2u, 0xa7179e84u, 0xbce6faadu, 0xffffffffu, 0xffffffffu, 0x00000000u, 0xffffffffu); }
  SG_HD static u256 R2() { return SG_U256(0xbe79eea2u, 0x83244c95u, 0x49bd6fa6u, 0x4699799cu, 0x2b6bec59u, 0x2845b239u, 0xf3d95620u, 0x66e12d94u); }
  SG_HD static u256 ONE_MONT() { return SG_U256(0x039cdaafu, 0x0c46353du, 0x58e8617bu, 0x43190552u, 0x00000000u, 0x00000000u, 0xffffffffu, 0x00000000u); }
  SG_HD static u256 N_MINUS_2() { return SG_U256(0xfc63254fu, 0xf3b9cac2u, 0xa7179e84u, 0xbce6faadu, 0xffffffffu, 0xffffffffu, 0x00000000u, 0xffffffffu); }
  static constexpr uint32_t NINV = 0xee00bc4fu;
  static constexpr uint32_t MINV30 = 0x11ff43b1u;
};

struct EdScalarC {
  SG_HD static u256 N() { return SG_U256(0x5cf5d3edu, 0x5812631au, 0xa2f79cd6u, 0x14def9deu, 0x00000000u, 0x00000000u, 0x00000000u, 0x10000000u); }
  SG_HD static u256 R2() { return SG_U256(0x449c0f01u, 0xa40611e3u, 0x68859347u, 0xd00e1ba7u, 0x17f5be65u, 0xceec73d2u, 0x7c309a3du, 0x0399411bu); }
  SG_HD static u256 ONE_MONT() { return SG_U256(0x8d98951du, 0xd6ec3174u, 0x737dcf70u, 0xc6ef5bf4u, 0xfffffffeu, 0xffffffffu, 0xffffffffu, 0x0fffffffu); }
  SG_HD static u256 N_MINUS_2() { return SG_U256(0x5cf5d3ebu, 0x5812631au, 0xa2f79cd6u, 0x14def9deu, 0x00000000u, 0x00000000u, 0x00000000u, 0x10000000u); }
  static constexpr uint32_t NINV = 0x12547e1bu;
  static constexpr uint32_t MINV30 = 0x2dab81e5u;
};

using ScK1 = Mont<K1ScalarC>;
using ScR1 = Mont<R1ScalarC>;
using ScEd = Mont<EdScalarC>;

// ---------------------------------------------------------------------------
// P-256 base field in Montgomery form (R = 2^256): a value a is held as
// a R mod p, weakly reduced (below 2^256).  p = 2^256 - 2^224 + 2^192 + 2^96 - 1
// is -1 mod 2^32, so -p^-1 = 1 mod 2^32 and each reduction round's quotient
// is the current low word q itself; q p = q 2^256 - q 2^224 + q 2^192 + q 2^96
// - q then cancels that word and adds q at words +3 and +6 and q (2^32 - 1)
// at words +7, +8 -- word-aligned additions, no multiplications (the
// structure OpenSSL's ecp_nistz256 uses with 64-bit words).  The reduction
// runs on the integer ALU while the products use the multiply pipe.
// ---------------------------------------------------------------------------
struct FpR1 {
  SG_HD static u256 P() { return SG_U256(0xffffffffu, 0xffffffffu, 0xffffffffu, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000001u, 0xffffffffu); }
  SG_HD static u256 R2() { return SG_U256(0x00000003u, 0x00000000u, 0xffffffffu, 0xfffffffbu, 0xfffffffeu, 0xffffffffu, 0xfffffffdu, 0x00000004u); }
  SG_HD static u256 R3() { return SG_U256(0x0000000au, 0xfffffffdu, 0xfffffff7u, 0xffffffedu, 0xfffffffcu, 0x00000005u, 0x00000001u, 0x00000018u); }

  // t 2^-256 mod p for t < 2^512, weakly reduced (below 2^256).  Round i adds
  // q p 2^(32 i) with q = t_i; its carry out of word i + 8 is held back and
  // added with the next round's high word (hi + carry < 2^32), so every round
  // is one carry chain over six words.  The sum (t + Q p) / 2^256 is below
  // 2^256 + p: a carry out of 2^256 is folded as K = 2^256 - p.
  SG_HD static u256 reduce(const uint32_t tin[16]) {
    uint32_t t[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) t[k] = tin[k];
    uint32_t c = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const uint32_t q = t[i];
      const uint32_t lo = sub_cc(0u, q);  // q (2^32 - 1) = hi 2^32 + lo
      const uint32_t hi = subc(q, 0u) + c;
      t[i + 3] = add_cc(t[i + 3], q);
      t[i + 4] = addc_cc(t[i + 4], 0u);
      t[i + 5] = addc_cc(t[i + 5], 0u);
      t[i + 6] = addc_cc(t[i + 6], q);
      t[i + 7] = addc_cc(t[i + 7], lo);
      t[i + 8] = addc_cc(t[i + 8], hi);
      c = addc(0u, 0u);
    }
    u256 r;
#pragma unroll
    for (int k = 0; k < 8; ++k) r.w[k] = t[8 + k];
    (void)add_k(r, c);  // r < p when c = 1, so r + K stays below 2^256
    return r;
  }

  SG_HD static u256 canon(const u256& x) { return reduce_once(x, P()); }  // x < 2^256 < 2p
  SG_HD static bool is_zero(const u256& a) { return u256_is_zero(a) || u256_eq(a, P()); }  // a == 0 mod p
  SG_NOINL static u256 mul(const u256 a, const u256 b) { uint32_t t[16]; mul_wide(t, a, b); return reduce(t); }
  SG_NOINL static u256 sqr(const u256 a) { uint32_t t[16]; sqr_wide(t, a); return reduce(t); }

  // t += c K with K = 2^256 - p = 2^224 - 2^192 - 2^96 + 1 (words 1, 0, 0,
  // 2^32 - 1 (three), 2^32 - 2, 0) for c in {0, 1}; returns the carry out
  SG_HD static uint32_t add_k(u256& t, uint32_t c) {
    const uint32_t m = 0u - c;
    t.w[0] = add_cc(t.w[0], c);
    t.w[1] = addc_cc(t.w[1], 0u);
    t.w[2] = addc_cc(t.w[2], 0u);
    t.w[3] = addc_cc(t.w[3], m);
    t.w[4] = addc_cc(t.w[4], m);
    t.w[5] = addc_cc(t.w[5], m);
    t.w[6] = addc_cc(t.w[6], m - c);
    t.w[7] = addc_cc(t.w[7], 0u);
    return addc(0u, 0u);
  }
  // t -= b K for b in {0, 1}; returns the borrow out
  SG_HD static uint32_t sub_k(u256& t, uint32_t b) {
    const uint32_t m = 0u - b;
    t.w[0] = sub_cc(t.w[0], b);
    t.w[1] = subc_cc(t.w[1], 0u);
    t.w[2] = subc_cc(t.w[2], 0u);
    t.w[3] = subc_cc(t.w[3], m);
    t.w[4] = subc_cc(t.w[4], m);
    t.w[5] = subc_cc(t.w[5], m);
    t.w[6] = subc_cc(t.w[6], m - b);
    t.w[7] = subc_cc(t.w[7], 0u);
    return subc(0u, 0u) & 1u;
  }
  // a + b for a, b < 2^256, weakly reduced: a carry out of 2^256 is worth K;
  // when adding K carries again the sum left is below K, so a second K
  // cannot carry
  SG_HD static u256 add(const u256& a, const u256& b) {
    u256 t;
    const uint32_t c = u256_add(t, a, b);
    (void)add_k(t, add_k(t, c));
    return t;
  }
  // a - b for a, b < 2^256, weakly reduced: a borrow is worth -K; after a
  // second borrow the value is at least p, so a second K cannot borrow
  SG_HD static u256 sub(const u256& a, const u256& b) {
    u256 t;
    const uint32_t bw = u256_sub(t, a, b);
    (void)sub_k(t, sub_k(t, bw));
    return t;
  }
  // a / 2 mod p for a < 2^256, weakly reduced: (a + p) / 2 when a is odd
  SG_HD static u256 half(const u256& a) {
    const uint32_t m = 0u - (a.w[0] & 1u);
    const u256 p = P();
    u256 t;
    t.w[0] = add_cc(a.w[0], p.w[0] & m);
#pragma unroll
    for (int j = 1; j < 8; ++j) t.w[j] = addc_cc(a.w[j], p.w[j] & m);
    const uint32_t c = addc(0u, 0u);
    u256 r;
#pragma unroll
    for (int j = 0; j < 7; ++j) r.w[j] = (t.w[j] >> 1) | (t.w[j + 1] << 31);
    r.w[7] = (t.w[7] >> 1) | (c << 31);
    return r;
  }
  SG_HD static u256 neg(const u256& a) { return sub(u256_zero(), a); }  // 0 - 0 = 0 without a borrow
  SG_HD static u256 one() { return SG_U256(0x00000001u, 0u, 0u, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xfffffffeu, 0u); }  // R mod p
  SG_HD static u256 zero() { return u256_zero(); }
  SG_HD static u256 from_int(const u256& x) { return mul(x, R2()); }  // any x < 2^256 -> x R mod p
  SG_HD static u256 to_int(const u256& a) {  // a R^-1 mod p, canonical
    uint32_t t[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) { t[k] = a.w[k]; t[8 + k] = 0u; }
    return canon(reduce(t));  // (a + Q p) / 2^256 <= p
  }
  // b R mod p
  SG_HD static u256 curve_b() { return SG_U256(0x29c4bddfu, 0xd89cdf62u, 0x78843090u, 0xacf005cdu, 0xf7212ed6u, 0xe5a220abu, 0x04874834u, 0xdc30061du); }

  SG_HD static u256 sqr_n(u256 a, int n) {
#pragma unroll 1
    for (int i = 0; i < n; ++i) a = sqr(a);
    return a;
  }

  // x2, x4, x8, x16, x32 blocks: a^(2^k - 1)
  SG_HD static void blocks(const u256 a, u256& x2, u256& x4, u256& x8, u256& x16, u256& x32) {
    x2 = mul(sqr(a), a);
    x4 = mul(sqr_n(x2, 2), x2);
    x8 = mul(sqr_n(x4, 4), x4);
    x16 = mul(sqr_n(x8, 8), x8);
    x32 = mul(sqr_n(x16, 16), x16);
  }

  // a^-1 by divsteps, verified; Fermat fallback.  The divsteps invert the
  // held value a R, so one Montgomery multiply by R^3 gives a^-1 R.
  SG_NOINL static u256 inv(const u256 a) {
    const u256 ac = canon(a);
    const u256 r = canon(mul(divstep_inverse(ac, P(), 0x3fffffffu), R3()));
    return u256_eq(canon(mul(ac, r)), one()) ? r : canon(inv_fermat(ac));
  }

  // a^(p-2), p-2 = ones[255..224] 0^31 1 0^96 ones[95..2] 0 1 : 255 S + 13 M
  SG_NOINL static u256 inv_fermat(const u256 a) {
    u256 x2, x4, x8, x16, x32;
    blocks(a, x2, x4, x8, x16, x32);
    u256 t = mul(sqr_n(x32, 32), a);
    t = sqr_n(t, 96);
    t = mul(sqr_n(t, 32), x32);
    t = mul(sqr_n(t, 32), x32);
    t = mul(sqr_n(t, 16), x16);
    t = mul(sqr_n(t, 8), x8);
    t = mul(sqr_n(t, 4), x4);
    t = mul(sqr_n(t, 2), x2);
    t = mul(sqr_n(t, 2), a);
    return t;
  }

  // a^((p+1)/4) = a^(2^254 - 2^222 + 2^190 + 2^94): 253 S + 7 M
  SG_NOINL static u256 sqrt_candidate(const u256 a) {
    u256 x2, x4, x8, x16, x32;
    blocks(a, x2, x4, x8, x16, x32);
    u256 t = mul(sqr_n(x32, 32), a);
    t = mul(sqr_n(t, 96), a);
    t = sqr_n(t, 94);
    return t;
  }
};

}  // namespace sg
