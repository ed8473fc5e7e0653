// 32-bit limb carry-chain primitives for sm_103a.
//
// Each primitive is one PTX instruction (add.cc / addc / mad.lo.cc / madc.hi
// ...), issued as its own `asm volatile` statement so that chains keep their
// program order; the PTX carry flag (CC.CF) links consecutive primitives.
// These replace the reference's 13-bit-limb WGSL bigint layer
// (src/wgsl/bigint.wgsl:1-246), whose u32-only arithmetic had no wide
// multiply and no carry flag.
//
// When compiled for the host (test builds only, never in libsigops.so's host
// code path) the carry flag is emulated with a thread-local word so that the
// device arithmetic can be checked against the oracle without a GPU.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define SG_HD __host__ __device__ __forceinline__
#define SG_DEV __device__ __forceinline__
// once-per-signature routines (exponentiation chains, scalar multiplication):
// compiled once and called, which keeps kernels small enough to compile fast
// (inline: a non-template one may sit in a header included by several units)
#define SG_NOINL inline __host__ __device__ __noinline__
#else
#define SG_HD inline
#define SG_DEV inline
#define SG_NOINL inline
#endif

namespace sg {

#if defined(__CUDA_ARCH__)

SG_DEV uint32_t add_cc(uint32_t a, uint32_t b) { uint32_t r; asm volatile("add.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r; }
SG_DEV uint32_t addc_cc(uint32_t a, uint32_t b) { uint32_t r; asm volatile("addc.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r; }
SG_DEV uint32_t addc(uint32_t a, uint32_t b) { uint32_t r; asm volatile("addc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r; }
SG_DEV uint32_t sub_cc(uint32_t a, uint32_t b) { uint32_t r; asm volatile("sub.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r; }
SG_DEV uint32_t subc_cc(uint32_t a, uint32_t b) { uint32_t r; asm volatile("subc.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r; }
SG_DEV uint32_t subc(uint32_t a, uint32_t b) { uint32_t r; asm volatile("subc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r; }
SG_DEV uint32_t mad_lo_cc(uint32_t a, uint32_t b, uint32_t c) { uint32_t r; asm volatile("mad.lo.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c)); return r; }
SG_DEV uint32_t madc_lo_cc(uint32_t a, uint32_t b, uint32_t c) { uint32_t r; asm volatile("madc.lo.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c)); return r; }
SG_DEV uint32_t madc_lo(uint32_t a, uint32_t b, uint32_t c) { uint32_t r; asm volatile("madc.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c)); return r; }
SG_DEV uint32_t mad_hi_cc(uint32_t a, uint32_t b, uint32_t c) { uint32_t r; asm volatile("mad.hi.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c)); return r; }
SG_DEV uint32_t madc_hi_cc(uint32_t a, uint32_t b, uint32_t c) { uint32_t r; asm volatile("madc.hi.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c)); return r; }
SG_DEV uint32_t madc_hi(uint32_t a, uint32_t b, uint32_t c) { uint32_t r; asm volatile("madc.hi.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c)); return r; }
SG_DEV uint32_t mul_lo(uint32_t a, uint32_t b) { return a * b; }
SG_DEV uint32_t mul_hi(uint32_t a, uint32_t b) { return __umulhi(a, b); }

// 32-bit multiply instructions of one operation (host test builds count them)
#define SG_COUNT_MULS(k) ((void)0)

#else  // host emulation (test builds)

inline uint32_t& cf_() { static thread_local uint32_t cf = 0; return cf; }
// multiply instructions executed by this thread: the work model of the kernels
// (a 32x32 -> 64-bit product is two: its low and its high half)
inline uint64_t& mulcount_() { static thread_local uint64_t c = 0; return c; }
#define SG_COUNT_MULS(k) (::sg::mulcount_() += (uint64_t)(k))
inline uint32_t add_cc(uint32_t a, uint32_t b) { uint64_t s = (uint64_t)a + b; cf_() = (uint32_t)(s >> 32); return (uint32_t)s; }
inline uint32_t addc_cc(uint32_t a, uint32_t b) { uint64_t s = (uint64_t)a + b + cf_(); cf_() = (uint32_t)(s >> 32); return (uint32_t)s; }
inline uint32_t addc(uint32_t a, uint32_t b) { return a + b + cf_(); }
inline uint32_t sub_cc(uint32_t a, uint32_t b) { uint64_t d = (uint64_t)a - b; cf_() = (uint32_t)(d >> 63); return (uint32_t)d; }
inline uint32_t subc_cc(uint32_t a, uint32_t b) { uint64_t d = (uint64_t)a - b - cf_(); cf_() = (uint32_t)(d >> 63); return (uint32_t)d; }
inline uint32_t subc(uint32_t a, uint32_t b) { return a - b - cf_(); }
inline uint32_t mad_lo_cc(uint32_t a, uint32_t b, uint32_t c) { ++mulcount_(); uint64_t s = (uint64_t)(uint32_t)(a * b) + c; cf_() = (uint32_t)(s >> 32); return (uint32_t)s; }
inline uint32_t madc_lo_cc(uint32_t a, uint32_t b, uint32_t c) { ++mulcount_(); uint64_t s = (uint64_t)(uint32_t)(a * b) + c + cf_(); cf_() = (uint32_t)(s >> 32); return (uint32_t)s; }
inline uint32_t madc_lo(uint32_t a, uint32_t b, uint32_t c) { ++mulcount_(); return (uint32_t)(a * b) + c + cf_(); }
inline uint32_t mad_hi_cc(uint32_t a, uint32_t b, uint32_t c) { ++mulcount_(); uint64_t s = (((uint64_t)a * b) >> 32) + c; cf_() = (uint32_t)(s >> 32); return (uint32_t)s; }
inline uint32_t madc_hi_cc(uint32_t a, uint32_t b, uint32_t c) { ++mulcount_(); uint64_t s = (((uint64_t)a * b) >> 32) + c + cf_(); cf_() = (uint32_t)(s >> 32); return (uint32_t)s; }
inline uint32_t madc_hi(uint32_t a, uint32_t b, uint32_t c) { ++mulcount_(); return (uint32_t)(((uint64_t)a * b) >> 32) + c + cf_(); }
inline uint32_t mul_lo(uint32_t a, uint32_t b) { ++mulcount_(); return a * b; }
inline uint32_t mul_hi(uint32_t a, uint32_t b) { ++mulcount_(); return (uint32_t)(((uint64_t)a * b) >> 32); }

#endif

SG_HD uint32_t bswap32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __byte_perm(x, 0, 0x0123);
#else
  return (x >> 24) | ((x >> 8) & 0xff00u) | ((x << 8) & 0xff0000u) | (x << 24);
#endif
}

// 256-bit unsigned integer, little-endian 32-bit limbs.
struct u256 {
  uint32_t w[8];
};

SG_HD u256 u256_zero() { u256 r; for (int i = 0; i < 8; ++i) r.w[i] = 0; return r; }
SG_HD u256 u256_small(uint32_t v) { u256 r = u256_zero(); r.w[0] = v; return r; }

SG_HD bool u256_is_zero(const u256& a) {
  uint32_t acc = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) acc |= a.w[i];
  return acc == 0;
}

SG_HD bool u256_eq(const u256& a, const u256& b) {
  uint32_t acc = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) acc |= a.w[i] ^ b.w[i];
  return acc == 0;
}

// r = a + b, returns the carry out (0/1)
SG_HD uint32_t u256_add(u256& r, const u256& a, const u256& b) {
  r.w[0] = add_cc(a.w[0], b.w[0]);
#pragma unroll
  for (int i = 1; i < 8; ++i) r.w[i] = addc_cc(a.w[i], b.w[i]);
  return addc(0u, 0u);
}

// r = a - b, returns the borrow out (0/1)
SG_HD uint32_t u256_sub(u256& r, const u256& a, const u256& b) {
  r.w[0] = sub_cc(a.w[0], b.w[0]);
#pragma unroll
  for (int i = 1; i < 8; ++i) r.w[i] = subc_cc(a.w[i], b.w[i]);
  return subc(0u, 0u) & 1u;
}

// a >= b
SG_HD bool u256_gte(const u256& a, const u256& b) {
  u256 t;
  return u256_sub(t, a, b) == 0;
}

SG_HD u256 u256_select(bool c, const u256& a, const u256& b) {  // c ? a : b
  u256 r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.w[i] = c ? a.w[i] : b.w[i];
  return r;
}

// 2N-limb product r = a * b of two N-limb values (N even).
// Row i adds b_i * a into two accumulators: `e` collects the products with even
// a-limbs (lo at column i+j, hi at i+j+1 for j even -- a contiguous run of N
// limbs), `o` those with odd a-limbs (a run starting at column i+1).  Each row
// is therefore one unbroken carry chain; the two are summed at the end.
template <int N>
SG_HD void mul_rows(uint32_t* r, const uint32_t* a, const uint32_t* b) {
  uint32_t e[2 * N], o[2 * N + 1];
  // row 0: plain products, no carries (e: columns 0..N-1, o: columns 1..N)
#pragma unroll
  for (int j = 0; j < N; j += 2) {
    e[j] = mul_lo(a[j], b[0]);
    e[j + 1] = mul_hi(a[j], b[0]);
    o[j + 1] = mul_lo(a[j + 1], b[0]);
    o[j + 2] = mul_hi(a[j + 1], b[0]);
  }
  e[N] = 0;
  o[N + 1] = 0;
#pragma unroll
  for (int i = 1; i < N; ++i) {
    const uint32_t bi = b[i];
    // even chain over columns i .. i+N-1; column i+N-1 holds the previous
    // row's carry and the carry out lands in the fresh column i+N
    e[i] = mad_lo_cc(a[0], bi, e[i]);
    e[i + 1] = madc_hi_cc(a[0], bi, e[i + 1]);
#pragma unroll
    for (int j = 2; j < N; j += 2) {
      e[i + j] = madc_lo_cc(a[j], bi, e[i + j]);
      e[i + j + 1] = madc_hi_cc(a[j], bi, e[i + j + 1]);
    }
    e[i + N] = addc(0u, 0u);
    // odd chain over columns i+1 .. i+N, carry out into the fresh column i+N+1
    o[i + 1] = mad_lo_cc(a[1], bi, o[i + 1]);
    o[i + 2] = madc_hi_cc(a[1], bi, o[i + 2]);
#pragma unroll
    for (int j = 3; j < N; j += 2) {
      o[i + j] = madc_lo_cc(a[j], bi, o[i + j]);
      o[i + j + 1] = madc_hi_cc(a[j], bi, o[i + j + 1]);
    }
    o[i + N + 1] = addc(0u, 0u);  // o[2N] is always 0: the product fits 2N limbs
  }
  // r = e + (o << 32)
  r[0] = e[0];
  r[1] = add_cc(e[1], o[1]);
#pragma unroll
  for (int k = 2; k < 2 * N; ++k) r[k] = addc_cc(e[k], o[k]);
}

// 512-bit product r[0..15] = a * b, schoolbook: 64 lo + 64 hi products.
SG_HD void mul_wide_school(uint32_t r[16], const u256& a, const u256& b) { mul_rows<8>(r, a.w, b.w); }

// 512-bit product r[0..15] = a * b, one level of subtractive Karatsuba over
// 128-bit halves (a = a1 2^128 + a0, b likewise):
//   a0 b1 + a1 b0 = a0 b0 + a1 b1 + (a0 - a1)(b1 - b0),
// with |a0 - a1| |b1 - b0| computed unsigned and its sign applied when the
// middle term is summed.  Three 128x128 products: 48 lo + 48 hi instead of
// 64 + 64 (high halves are the costly multiply), for ~45 more add/select ops.
SG_HD void mul_wide_kara(uint32_t r[16], const u256& a, const u256& b) {
  uint32_t p0[8], p2[8], m[8], da[4], db[4], t[4];
  mul_rows<4>(p0, a.w, b.w);
  mul_rows<4>(p2, a.w + 4, b.w + 4);
  // da = |a0 - a1|, sa = all-ones when a0 < a1
  da[0] = sub_cc(a.w[0], a.w[4]);
#pragma unroll
  for (int k = 1; k < 4; ++k) da[k] = subc_cc(a.w[k], a.w[4 + k]);
  const uint32_t sa = subc(0u, 0u);
  t[0] = sub_cc(a.w[4], a.w[0]);
#pragma unroll
  for (int k = 1; k < 4; ++k) t[k] = subc_cc(a.w[4 + k], a.w[k]);
#pragma unroll
  for (int k = 0; k < 4; ++k) da[k] = sa ? t[k] : da[k];
  // db = |b1 - b0|, sb = all-ones when b1 < b0
  db[0] = sub_cc(b.w[4], b.w[0]);
#pragma unroll
  for (int k = 1; k < 4; ++k) db[k] = subc_cc(b.w[4 + k], b.w[k]);
  const uint32_t sb = subc(0u, 0u);
  t[0] = sub_cc(b.w[0], b.w[4]);
#pragma unroll
  for (int k = 1; k < 4; ++k) t[k] = subc_cc(b.w[k], b.w[4 + k]);
#pragma unroll
  for (int k = 0; k < 4; ++k) db[k] = sb ? t[k] : db[k];
  mul_rows<4>(m, da, db);
  // mid = p0 + p2 + (-1)^neg m, 9 limbs (its value is a0 b1 + a1 b0 < 2^257);
  // the negative case adds ~m + 1 over 9 limbs, the +1 entering as the carry
  const uint32_t neg = sa ^ sb;
  uint32_t mid[9];
  mid[0] = add_cc(p0[0], p2[0]);
#pragma unroll
  for (int k = 1; k < 8; ++k) mid[k] = addc_cc(p0[k], p2[k]);
  mid[8] = addc(0u, 0u);
  (void)add_cc(neg & 1u, 0xffffffffu);  // carry flag = neg
#pragma unroll
  for (int k = 0; k < 8; ++k) mid[k] = addc_cc(mid[k], m[k] ^ neg);
  mid[8] = addc(mid[8], neg);
  // r = p0 + mid 2^128 + p2 2^256
#pragma unroll
  for (int k = 0; k < 4; ++k) r[k] = p0[k];
  r[4] = add_cc(p0[4], mid[0]);
#pragma unroll
  for (int k = 5; k < 8; ++k) r[k] = addc_cc(p0[k], mid[k - 4]);
#pragma unroll
  for (int k = 8; k < 13; ++k) r[k] = addc_cc(p2[k - 8], mid[k - 4]);
  r[13] = addc_cc(p2[5], 0u);
  r[14] = addc_cc(p2[6], 0u);
  r[15] = addc(p2[7], 0u);
}

// the 512-bit product of the secp256k1 / P-256 / scalar-field multiplications
// (ed25519 uses mul_wide_kara)
SG_HD void mul_wide(uint32_t r[16], const u256& a, const u256& b) { mul_wide_school(r, a, b); }

// 512-bit square r[0..15] = a^2: the 28 cross products a_i a_j (i < j) are
// accumulated with the same even/odd single-chain rows as mul_wide (row i
// covers j > i only), doubled by a one-bit shift, then the 8 diagonal squares
// are added in one chain: 72 multiply instructions instead of 128.
SG_HD void sqr_wide(uint32_t r[16], const u256& a) {
  uint32_t e[16], o[16];
  // row 0 (plain products): even j = 2,4,6 -> e[2..7]; odd j = 1,3,5,7 -> o[1..8]
  e[0] = 0;
  e[1] = 0;
#pragma unroll
  for (int j = 2; j < 8; j += 2) {
    e[j] = mul_lo(a.w[j], a.w[0]);
    e[j + 1] = mul_hi(a.w[j], a.w[0]);
  }
#pragma unroll
  for (int j = 1; j < 8; j += 2) {
    o[j] = mul_lo(a.w[j], a.w[0]);
    o[j + 1] = mul_hi(a.w[j], a.w[0]);
  }
  e[8] = 0;
  o[9] = 0;
#pragma unroll
  for (int i = 1; i < 7; ++i) {
    const uint32_t bi = a.w[i];
    // even chain: even j > i, columns [i + j0, i + 7], carry into fresh column i + 8
    const int j0 = (i & 1) ? i + 1 : i + 2;
    if (j0 <= 6) {
#pragma unroll
      for (int j = j0; j <= 6; j += 2) {
        e[i + j] = (j == j0) ? mad_lo_cc(a.w[j], bi, e[i + j]) : madc_lo_cc(a.w[j], bi, e[i + j]);
        e[i + j + 1] = madc_hi_cc(a.w[j], bi, e[i + j + 1]);
      }
      e[i + 8] = addc(0u, 0u);
    } else {
      e[i + 8] = 0;
    }
    // odd chain: odd j > i, columns [i + j1, i + 8], carry into fresh column i + 9
    const int j1 = (i & 1) ? i + 2 : i + 1;
#pragma unroll
    for (int j = j1; j <= 7; j += 2) {
      o[i + j] = (j == j1) ? mad_lo_cc(a.w[j], bi, o[i + j]) : madc_lo_cc(a.w[j], bi, o[i + j]);
      o[i + j + 1] = madc_hi_cc(a.w[j], bi, o[i + j + 1]);
    }
    if (i + 9 < 16) o[i + 9] = addc(0u, 0u);
  }
  e[15] = 0;
  // c = e + o (column-aligned), then r = 2c + diagonal
  uint32_t c[16];
  c[0] = 0;
  c[1] = add_cc(e[1], o[1]);
#pragma unroll
  for (int k = 2; k < 16; ++k) c[k] = addc_cc(e[k], o[k]);
  uint32_t d[16];
  d[0] = c[0] << 1;
#pragma unroll
  for (int k = 1; k < 16; ++k) d[k] = (c[k] << 1) | (c[k - 1] >> 31);
  r[0] = mad_lo_cc(a.w[0], a.w[0], d[0]);
  r[1] = madc_hi_cc(a.w[0], a.w[0], d[1]);
#pragma unroll
  for (int i = 1; i < 8; ++i) {
    r[2 * i] = madc_lo_cc(a.w[i], a.w[i], d[2 * i]);
    r[2 * i + 1] = (i < 7) ? madc_hi_cc(a.w[i], a.w[i], d[2 * i + 1]) : madc_hi(a.w[i], a.w[i], d[2 * i + 1]);
  }
}

}  // namespace sg
