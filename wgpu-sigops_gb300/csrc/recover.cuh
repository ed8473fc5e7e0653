// One signature: secp256k1 / P-256 public-key recovery and ed25519
// verification, written once for the plain kernels, the batched kernel and the
// host-side test build.
//
// Inputs and outputs are u32 words exactly as the bytes sit in memory
// (little-endian loads): signatures 16 words, messages and keys 8 words.
#pragma once
#include "curve.cuh"
#include "sha512.cuh"

namespace sg {

// per-item status (include/sigops.h SIGOPS_ST_*)
enum : uint8_t { ST_OK = 0, ST_BAD_SCALAR = 1, ST_NO_POINT = 2, ST_INFINITY = 3, ST_MISMATCH = 4 };

// 32 big-endian bytes (as 8 loaded words) -> integer
SG_HD u256 be_words_to_u256(const uint32_t* w) {
  u256 r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.w[i] = bswap32(w[7 - i]);
  return r;
}
SG_HD void u256_to_be_words(const u256& v, uint32_t* w) {
#pragma unroll
  for (int i = 0; i < 8; ++i) w[7 - i] = bswap32(v.w[i]);
}

// ---------------------------------------------------------------------------
// ECDSA recovery
// ---------------------------------------------------------------------------
// Window widths of the signed fixed windows (Booth): the per-signature point R
// uses multiples 1..2^(WR-1) built per thread; the generator uses a
// precomputed table of multiples 1..2^(WG-1).  The defaults: WR = 5 and WG =
// 16, a table in global memory (2 MiB, read through the read-only path and
// resident in L2), so that a 256-bit scalar costs 17 generator additions
// instead of 33 with 8-bit windows.  The batched engine also compiles WR = 4
// and 6, and WG = 8 with its 128-entry tables staged into shared memory by a
// bulk (TMA) copy; the autotuner times them.
constexpr int ECDSA_WR = 5;
constexpr int ECDSA_WG = 16;
constexpr int ECDSA_GTAB = 1 << (ECDSA_WG - 1);  // 32768 affine points
constexpr int ED_WR = 5;
constexpr int ED_WG = 16;
constexpr int ED_GTAB = 1 << (ED_WG - 1);  // 32768 affine Niels points
constexpr int SMALL_WG = 8;                      // generator windows of tables staged in shared memory
constexpr int SMALL_GTAB = 1 << (SMALL_WG - 1);  // 128 entries

struct K1Traits {
  using F = FpK1;
  using S = ScK1;
  static constexpr bool A_M3 = false;
  SG_HD static u256 rhs(const u256& x) { return F::add(F::mul(F::sqr(x), x), u256_small(7)); }
};
struct R1Traits {
  using F = FpR1;
  using S = ScR1;
  static constexpr bool A_M3 = true;
  SG_HD static u256 rhs(const u256& x) {
    u256 x3 = F::mul(F::sqr(x), x);
    u256 x3a = F::sub(x3, F::add(F::add(x, x), x));
    return F::add(x3a, F::curve_b());
  }
};

// n words of a table in global memory (16-byte aligned), read-only path
SG_HD void load_table_words(const uint32_t* e, int n, uint32_t* w) {
#ifdef __CUDA_ARCH__
  const uint4* q = reinterpret_cast<const uint4*>(e);
#pragma unroll
  for (int k = 0; k < n / 4; ++k) {
    const uint4 v = __ldg(q + k);
    w[4 * k] = v.x;
    w[4 * k + 1] = v.y;
    w[4 * k + 2] = v.z;
    w[4 * k + 3] = v.w;
  }
#else
  for (int k = 0; k < n; ++k) w[k] = e[k];
#endif
}

// n words of a table staged in shared memory (16-byte aligned)
SG_HD void load_smem_words(const uint32_t* e, int n, uint32_t* w) {
#ifdef __CUDA_ARCH__
  const uint4* q = reinterpret_cast<const uint4*>(e);
#pragma unroll
  for (int k = 0; k < n / 4; ++k) {
    const uint4 v = q[k];
    w[4 * k] = v.x;
    w[4 * k + 1] = v.y;
    w[4 * k + 2] = v.z;
    w[4 * k + 3] = v.w;
  }
#else
  for (int k = 0; k < n; ++k) w[k] = e[k];
#endif
}

// entry idx of a generator table: global memory for 16-bit windows, shared
// memory for the small tables
template <int WG = ECDSA_WG>
SG_HD APoint load_apoint(const uint32_t* t, uint32_t idx) {
  uint32_t w[16];
  if constexpr (WG == ECDSA_WG) load_table_words(t + (size_t)idx * 16u, 16, w);
  else load_smem_words(t + (size_t)idx * 16u, 16, w);
  APoint a;
#pragma unroll
  for (int k = 0; k < 8; ++k) { a.x.w[k] = w[k]; a.y.w[k] = w[8 + k]; }
  return a;
}

// The per-signature table of multiples 1..NR of R, affine, so that every
// R-side addition of the doubling chain is a mixed addition (8M + 3S instead
// of 11M + 5S).  Built with co-Z additions (Meloni, "New point addition
// formulae for ECC applications", WAIFI 2007): 2R comes from the doubling of
// an affine point that also returns R at 2R's Z (1M + 5S), then
// (k+1)R = R' + kR with R' kept at kR's Z (4M + 2S, against 8M + 3S for a
// mixed addition).  Each such step multiplies the common Z by
// d_k = X(R') - X(kR), so the table is made affine with one inversion of the
// last Z followed by Z_k^-1 = Z_(k+1)^-1 d_(k+1) down the chain (no prefix
// products).  No step meets an exceptional case: R has prime order above NR,
// so kR != +-R for 2 <= k <= NR - 1 and R.y != 0.
//
// coz_chain builds the entries, tab[k] at its own Z_k = dz[1] ... dz[k]
// (Z_0 = 1); coz_table makes them affine, coz_table_iso brings them to the
// last Z without an inversion.
template <class F, bool A_M3, int NR>
SG_HD void coz_chain(const APoint R, APoint* tab, u256* dz) {
  // dz[1] = Z(2R); dz[k] = Z(tab[k]) / Z(tab[k-1]) for k >= 2
  const u256 B = F::sqr(R.x);
  const u256 E = F::sqr(R.y);
  const u256 L = F::sqr(E);
  u256 S = F::sub(F::sub(F::sqr(F::add(R.x, E)), B), L);
  S = F::add(S, S);                               // 4 x y^2 = X(R') at Z = 2y
  u256 M = A_M3 ? F::sub(B, F::one()) : B;        // 3 x^2 + a
  M = F::add(F::add(M, M), M);
  u256 L8 = F::add(L, L);
  L8 = F::add(L8, L8);
  L8 = F::add(L8, L8);                            // 8 y^4 = Y(R') at Z = 2y
  tab[0] = R;
  tab[1].x = F::sub(F::sqr(M), F::add(S, S));
  tab[1].y = F::sub(F::mul(M, F::sub(S, tab[1].x)), L8);
  dz[1] = F::add(R.y, R.y);
  u256 px = S, py = L8;
#pragma unroll 1
  for (int k = 2; k < NR; ++k) {
    const u256 d = F::sub(px, tab[k - 1].x);
    const u256 e = F::sub(py, tab[k - 1].y);
    const u256 C = F::sqr(d);
    const u256 W1 = F::mul(px, C);
    const u256 W2 = F::mul(tab[k - 1].x, C);
    const u256 A1 = F::mul(py, F::sub(W1, W2));
    tab[k].x = F::sub(F::sub(F::sqr(e), W1), W2);
    tab[k].y = F::sub(F::mul(e, F::sub(W1, tab[k].x)), A1);
    dz[k] = d;
    px = W1;
    py = A1;
  }
}

template <class F, bool A_M3, int NR>
SG_HD void coz_table(const APoint R, APoint* tab) {
  u256 dz[NR];
  coz_chain<F, A_M3, NR>(R, tab, dz);
  u256 z = dz[1];
#pragma unroll 1
  for (int k = 2; k < NR; ++k) z = F::mul(z, dz[k]);
  u256 inv = F::inv(z);
#pragma unroll 1
  for (int k = NR - 1; k >= 1; --k) {
    const u256 z2 = F::sqr(inv);
    tab[k].x = F::mul(tab[k].x, z2);
    tab[k].y = F::mul(tab[k].y, F::mul(z2, inv));
    if (k > 1) inv = F::mul(inv, dz[k]);
  }
}

// The same multiples for a curve with a = 0, without the inversion: every
// entry is brought to the chain's last Z, zc = Z_(NR-1), by s_k = zc / Z_k =
// dz[k+1] ... dz[NR-1] (X s_k^2, Y s_k^3).  The entries are then affine points
// of the isomorphic curve E': y^2 = x^3 + b zc^6, the image of E under
// psi(x, y) = (zc^2 x, zc^3 y).  With a = 0 neither the doubling nor the
// additions read a curve constant, so a chain on E' runs the same formulas;
// a point of E added into it enters as psi(P) (two multiplications), and a
// Jacobian result (X, Y, Z) on E' is (X, Y, Z zc) on E.  Against coz_table
// this saves the inversion and the product of the dz (NR-2 multiplications)
// and costs the same per entry.  psi commutes with negation and with
// phi(x, y) = (beta x, y).  NR >= 2.
template <class F, int NR>
SG_HD void coz_table_iso(const APoint R, APoint* tab, u256& zc) {
  u256 dz[NR];
  coz_chain<F, false, NR>(R, tab, dz);
  u256 sk = dz[NR - 1];  // s_(NR-2)
#pragma unroll 1
  for (int k = NR - 2;; --k) {
    const u256 s2 = F::sqr(sk);
    tab[k].x = F::mul(tab[k].x, s2);
    tab[k].y = F::mul(tab[k].y, F::mul(s2, sk));
    if (k == 0) break;
    sk = F::mul(sk, dz[k]);
  }
  zc = sk;  // s_0 = Z_(NR-1) / Z_0
}

// psi(P) for P affine on E, zc2 = zc^2, zc3 = zc^3 (see coz_table_iso)
template <class F>
SG_HD APoint iso_point(const APoint& p, const u256& zc2, const u256& zc3) {
  APoint r;
  r.x = F::mul(p.x, zc2);
  r.y = F::mul(p.y, zc3);
  return r;
}

// u1 * G + u2 * R, signed fixed windows, one shared doubling chain.
// gtab: multiples 1..2^(WG-1) of G, affine, field representation.
template <class T, int WR = ECDSA_WR, int WG = ECDSA_WG>
SG_NOINL JPoint ecdsa_lincomb(const u256 u1, const u256 u2, const APoint R, const uint32_t* gtab) {
  using W = Weier<typename T::F, T::A_M3>;
  constexpr int NR = 1 << (WR - 1);
  APoint tab[NR];
  coz_table<typename T::F, T::A_M3, NR>(R, tab);

  constexpr int JR = (257 + WR - 1) / WR;  // windows for a 256-bit scalar
  constexpr int JG = (257 + WG - 1) / WG;
  // the chain starts at the highest window position that adds anything:
  // doublings above it would only double the point at infinity
  constexpr int TOP = ((JR - 1) * WR > (JG - 1) * WG) ? (JR - 1) * WR : (JG - 1) * WG;
  JPoint acc = W::infinity();
#pragma unroll 1
  for (int pos = TOP; pos >= 0; --pos) {
    // the generator entry is read before the doubling, which hides the read
    bool gneg = false;
    uint32_t gd = 0;
    APoint ge;
    if (pos % WG == 0) {
      gd = booth_digit(u1, pos / WG, WG, gneg);
      if (gd) ge = load_apoint<WG>(gtab, gd - 1);
    }
    acc = W::dbl(acc);
    // u2 R's then u1 G's window through one addition site (one copy of the
    // mixed addition in the loop: see k1_glv_lincomb)
    const uint32_t first = pos % WR == 0 ? 0u : 1u;
    const uint32_t last = pos % WG == 0 ? 2u : 1u;
#pragma unroll 1
    for (uint32_t src = first; src < last; ++src) {
      bool neg = gneg;
      const uint32_t d = src == 0 ? booth_digit(u2, pos / WR, WR, neg) : gd;
      if (!d) continue;
      APoint e;
      if (src == 0) e = tab[d - 1];
      else e = ge;
      if (neg) e = W::neg(e);
      acc = W::madd(acc, e);
    }
  }
  return acc;
}

// ---------------------------------------------------------------------------
// secp256k1 with the GLV endomorphism phi(x, y) = (beta x, y) = lambda (x, y):
// u2 R = k1 R + k2 phi(R) with |k1|, |k2| < 2^128 and u1 G = a G + b (2^128 G)
// (a, b the two 128-bit halves of u1), so the shared doubling chain is ~133
// doublings instead of ~260.  Decomposition constants as in the reference's
// src/curve_algos/secp256k1_curve.rs:47-71 (Babai rounding with g1, g2 scaled
// by 2^384); the CPU model of GLV is src/curve_algos/secp256k1_mul.rs:38-94.
// gtab2: multiples 1..2^(WG-1) of G followed by the same multiples of 2^128 G.
// ---------------------------------------------------------------------------
struct K1Glv {
  SG_HD static u256 LAMBDA_MONT() { return SG_U256(0xc9926c9eu, 0xf07deb3du, 0x83c6944cu, 0x2c93e7adu, 0x52697d91u, 0x73a96606u, 0x8558d639u, 0x53284017u); }
  SG_HD static u256 BETA() { return SG_U256(0x719501eeu, 0xc1396c28u, 0x12f58995u, 0x9cf04975u, 0xac3434e9u, 0x6e64479eu, 0x657c0710u, 0x7ae96a2bu); }
  SG_HD static u256 G1() { return SG_U256(0x45dbb031u, 0xe893209au, 0x71e8ca7fu, 0x3daa8a14u, 0x9284eb15u, 0xe86c90e4u, 0xa7d46bcdu, 0x3086d221u); }
  SG_HD static u256 G2() { return SG_U256(0x8ac47f71u, 0x1571b4aeu, 0x9df506c6u, 0x221208acu, 0x0abfe4c4u, 0x6f547fa9u, 0x010e8828u, 0xe4437ed6u); }
  SG_HD static u256 MINUS_B1() { return SG_U256(0x0abfe4c3u, 0x6f547fa9u, 0x010e8828u, 0xe4437ed6u, 0u, 0u, 0u, 0u); }
  SG_HD static u256 B2() { return SG_U256(0x9284eb15u, 0xe86c90e4u, 0xa7d46bcdu, 0x3086d221u, 0u, 0u, 0u, 0u); }
  SG_HD static u256 HALF_N() { return SG_U256(0x681b20a0u, 0xdfe92f46u, 0x57a4501du, 0x5d576e73u, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0x7fffffffu); }

  // round(k * g / 2^384) for k < 2^256, g < 2^256: bits 384..511 plus bit 383
  SG_HD static u256 mul_shift384(const u256& k, const u256& g) {
    uint32_t t[16];
    mul_wide(t, k, g);
    u256 r = u256_zero();
    r.w[0] = add_cc(t[12], t[11] >> 31);
    r.w[1] = addc_cc(t[13], 0u);
    r.w[2] = addc_cc(t[14], 0u);
    r.w[3] = addc_cc(t[15], 0u);
    r.w[4] = addc(0u, 0u);
    return r;
  }

  // product of two values below 2^129, reduced mod n (fits 256 bits + reduce_once)
  SG_HD static u256 mul_small_mod_n(const u256& a, const u256& b) {
    uint32_t t[16];
    mul_wide(t, a, b);
    u256 r;
#pragma unroll
    for (int k = 0; k < 8; ++k) r.w[k] = t[k];
    return reduce_once(r, K1ScalarC::N());
  }

  // k = k1 + k2 lambda (mod n); returns |k1|, |k2| and their signs
  SG_HD static void split(const u256& k, u256& k1, bool& neg1, u256& k2, bool& neg2) {
    const u256 N = K1ScalarC::N();
    u256 c1 = mul_shift384(k, G1());
    u256 c2 = mul_shift384(k, G2());
    u256 r2 = mod_sub(mul_small_mod_n(c1, MINUS_B1()), mul_small_mod_n(c2, B2()), N);
    u256 r1 = mod_sub(k, ScK1::mul(r2, LAMBDA_MONT()), N);  // Montgomery: r2 * (lambda R) / R
    u256 t;
    neg1 = u256_gte(HALF_N(), r1) == false;
    u256_sub(t, N, r1);
    k1 = neg1 ? t : r1;
    neg2 = u256_gte(HALF_N(), r2) == false;
    u256_sub(t, N, r2);
    k2 = neg2 ? t : r2;
  }
};

template <int WR = ECDSA_WR, int WG = ECDSA_WG>
SG_NOINL JPoint k1_glv_lincomb(const u256 u1, const u256 u2, const APoint R, const uint32_t* gtab2) {
  using F = FpK1;
  using W = Weier<F, false>;
  constexpr int NR = 1 << (WR - 1);
  constexpr int HALF = 1 << (WG - 1);  // entries per half of the table
  u256 k1, k2;
  bool neg1, neg2;
  K1Glv::split(u2, k1, neg1, k2, neg2);
  APoint R1 = neg1 ? W::neg(R) : R;
  APoint tab[NR];
  u256 zc;  // the chain runs on E' (coz_table_iso); generator entries enter as psi(P)
  coz_table_iso<F, NR>(R1, tab, zc);
  const u256 zc2 = F::sqr(zc);
  const u256 zc3 = F::mul(zc2, zc);
  // phi(+-R) multiples: (beta x, +-y); k2's sign relative to k1's
  const bool flip2 = neg1 != neg2;
  const u256 beta = K1Glv::BETA();
  u256 a = u1, b = u256_zero();
#pragma unroll
  for (int k = 0; k < 4; ++k) { b.w[k] = u1.w[4 + k]; a.w[4 + k] = 0; }

  constexpr int JR = (130 + WR - 1) / WR;  // windows for a 129-bit magnitude
  constexpr int JG = (129 + WG - 1) / WG;  // windows for a 128-bit half
  // the chain starts at the highest window position that adds anything:
  // doublings above it would only double the point at infinity
  constexpr int TOP = ((JR - 1) * WR > (JG - 1) * WG) ? (JR - 1) * WR : (JG - 1) * WG;
  JPoint acc = W::infinity();
#pragma unroll 1
  for (int pos = TOP; pos >= 0; --pos) {
    acc = W::dbl(acc);
    // the window additions at this position, in the order k1 R, k2 phi(R),
    // a G, b 2^128 G, through one addition site: one copy of the mixed
    // addition in the loop instead of four keeps the loop's code small
    // enough for the instruction cache when warps run different phases
    const uint32_t first = pos % WR == 0 ? 0u : 2u;
    const uint32_t last = pos % WG == 0 ? 4u : 2u;
#pragma unroll 1
    for (uint32_t src = first; src < last; ++src) {
      const bool rs = src < 2;
      const u256 k = src == 0 ? k1 : src == 1 ? k2 : src == 2 ? a : b;
      bool ng;
      const uint32_t d = rs ? booth_digit(k, pos / WR, WR, ng) : booth_digit(k, pos / WG, WG, ng);
      if (!d) continue;
      APoint e;
      if (rs) {
        e = tab[d - 1];
        if (src == 1) e.x = F::mul(e.x, beta);
      } else {
        e = iso_point<F>(load_apoint<WG>(gtab2, (src == 3 ? (uint32_t)HALF : 0u) + d - 1), zc2, zc3);
      }
      if (ng != (src == 1 && flip2)) e = W::neg(e);
      acc = W::madd(acc, e);
    }
  }
  if (!W::is_inf(acc)) acc.Z = F::mul(acc.Z, zc);  // back to E; infinity keeps Z exactly 0
  return acc;
}

// Decode a fuel-encoded signature (recovery parity in bit 7 of s[0]) and
// recover R, with the validity rules of libsecp256k1 / p256 recovery: r, s in
// [1, n-1], z = msg mod n, a checked square root for R.y.  Follows the
// reference's one-kernel path (src/wgsl/secp256k1_ecdsa.wgsl:87-130,
// src/wgsl/secp256r1_ecdsa.wgsl:87-130).  Returns ST_OK or the item's status.
template <class T>
SG_HD uint8_t ecdsa_prepare(const uint32_t sig[16], const uint32_t msg[8], u256& r, u256& s, u256& z, APoint& R) {
  using F = typename T::F;
  using S = typename T::S;
  const u256 N = S::N();
  r = be_words_to_u256(sig);
  uint32_t sw[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) sw[k] = sig[8 + k];
  const uint32_t parity = (sw[0] >> 7) & 1u;  // byte 32 is the low byte of word 8
  sw[0] &= 0xffffff7fu;
  s = be_words_to_u256(sw);
  z = reduce_once(be_words_to_u256(msg), N);
  if (u256_is_zero(r) || u256_gte(r, N) || u256_is_zero(s) || u256_gte(s, N)) return ST_BAD_SCALAR;

  // R = (r, y) with y^2 = r^3 + a r + b and the requested parity
  u256 x = F::from_int(r);
  u256 rhs = T::rhs(x);
  u256 y = F::sqrt_candidate(rhs);
  if (!u256_eq(F::canon(F::sqr(y)), F::canon(rhs))) return ST_NO_POINT;
  if ((F::to_int(y).w[0] & 1u) != parity) y = F::neg(y);
  R.x = x;
  R.y = y;
  return ST_OK;
}

// Q = (-z / r) G + (s / r) R for a prepared signature, rinv_m = r^-1 in the
// scalar field's Montgomery form; ST_INFINITY when Q is the point at infinity
template <class T, bool GLV, int WR = ECDSA_WR, int WG = ECDSA_WG>
SG_HD uint8_t ecdsa_key_jacobian(const u256& s, const u256& z, const APoint& R, const u256& rinv_m, const uint32_t* gtab, JPoint& Q) {
  using S = typename T::S;
  using W = Weier<typename T::F, T::A_M3>;
  const u256 u2 = S::mul(s, rinv_m);
  const u256 u1 = S::neg(S::mul(z, rinv_m));
  if constexpr (GLV) Q = k1_glv_lincomb<WR, WG>(u1, u2, R, gtab);
  else Q = ecdsa_lincomb<T, WR, WG>(u1, u2, R, gtab);
  return W::is_inf(Q) ? ST_INFINITY : ST_OK;
}

// Recover the signer's key: out = x || y big-endian (zero unless ST_OK).
template <class T, bool GLV = false>
SG_HD uint8_t ecdsa_recover(const uint32_t sig[16], const uint32_t msg[8], const uint32_t* gtab, uint32_t out[16]) {
  using F = typename T::F;
  using S = typename T::S;
  using W = Weier<F, T::A_M3>;
#pragma unroll
  for (int k = 0; k < 16; ++k) out[k] = 0;
  u256 r, s, z;
  APoint R;
  uint8_t st = ecdsa_prepare<T>(sig, msg, r, s, z, R);
  if (st != ST_OK) return st;
  const u256 rinv_m = S::from_int(S::inv_int(r));  // r^-1 in Montgomery form
  JPoint Q;
  st = ecdsa_key_jacobian<T, GLV>(s, z, R, rinv_m, gtab, Q);
  if (st != ST_OK) return st;
  APoint a = W::to_affine(Q);
  u256_to_be_words(F::to_int(a.x), out);
  u256_to_be_words(F::to_int(a.y), out + 8);
  return ST_OK;
}

// r of a signature as the factor of the batched engine's simultaneous
// inversion: r in Montgomery form when r is in [1, n-1], else one (such an
// item fails its range check and never uses its inverse)
template <class T>
SG_HD u256 ecdsa_r_factor(const uint32_t sig[16]) {
  using S = typename T::S;
  const u256 r = be_words_to_u256(sig);
  const bool ok = !u256_is_zero(r) && !u256_gte(r, S::N());
  return ok ? S::from_int(r) : S::one();
}

// Montgomery's simultaneous inversion of v[0 .. m) in place (m >= 1, every
// v[j] invertible): prefix products, one inversion of their product,
// back-substitution -- 3 (m - 1) multiplications and one inversion for m
// inverses.  pre: scratch of m entries.  inv_one inverts a single value.
template <class Fd, class Inv>
SG_HD void batch_invert(u256* v, u256* pre, int m, Inv inv_one) {
  pre[0] = v[0];
#pragma unroll 1
  for (int j = 1; j < m; ++j) pre[j] = Fd::mul(pre[j - 1], v[j]);
  u256 inv = inv_one(pre[m - 1]);
#pragma unroll 1
  for (int j = m - 1; j > 0; --j) {
    const u256 vj = v[j];
    v[j] = Fd::mul(inv, pre[j - 1]);
    inv = Fd::mul(inv, vj);
  }
  v[0] = inv;
}

// the affine key of a Jacobian point given Z^-1, as 16 big-endian words
template <class T>
SG_HD void ecdsa_encode_key(const JPoint& Q, const u256& zi, uint32_t out[16]) {
  using F = typename T::F;
  const u256 zi2 = F::sqr(zi);
  u256_to_be_words(F::to_int(F::mul(Q.X, zi2)), out);
  u256_to_be_words(F::to_int(F::mul(Q.Y, F::mul(zi2, zi))), out + 8);
}

// ---------------------------------------------------------------------------
// ed25519 verification (ed25519-dalek 2.1.1 VerifyingKey::verify semantics)
// ---------------------------------------------------------------------------
template <int WG = ED_WG>
SG_HD EAffNiels load_eniels(const uint32_t* t, uint32_t idx) {
  uint32_t w[24];
  if constexpr (WG == ED_WG) load_table_words(t + (size_t)idx * 24u, 24, w);
  else load_smem_words(t + (size_t)idx * 24u, 24, w);
  EAffNiels a;
#pragma unroll
  for (int k = 0; k < 8; ++k) { a.ypx.w[k] = w[k]; a.ymx.w[k] = w[8 + k]; a.t2d.w[k] = w[16 + k]; }
  return a;
}

// 64-byte little-endian digest mod l (src/wgsl/ed25519_reduce_fr.wgsl:88-125)
SG_HD u256 reduce512_mod_l(const uint32_t h[16]) {
  u256 lo, hi;
#pragma unroll
  for (int k = 0; k < 8; ++k) { lo.w[k] = h[k]; hi.w[k] = h[8 + k]; }
  // (lo + hi * 2^256) * R mod l, then out of Montgomery form
  const u256 R3 = SG_U256(0x7b83a2dbu, 0x2a9e4968u, 0xaef7f3ecu, 0x278324e6u, 0x04ec5b65u, 0x8065dc6cu, 0x3599cec7u, 0x0e530b77u);
  u256 t = ScEd::add(ScEd::mul(hi, R3), ScEd::from_int(lo));
  return ScEd::to_int(t);
}

// k = SHA-512(R || A || M) mod l
SG_HD u256 ed_challenge(const uint32_t sig[16], const uint32_t pk[8], const uint32_t msg[8]) {
  uint32_t m[24], h[16];
#pragma unroll
  for (int k = 0; k < 8; ++k) { m[k] = sig[k]; m[8 + k] = pk[k]; m[16 + k] = msg[k]; }
  sha512_96(m, h);
  return reduce512_mod_l(h);
}

// [s]B + [k](-A), signed fixed windows; btab: multiples 1..2^(WG-1) of B (affine Niels)
template <int WR = ED_WR, int WG = ED_WG>
SG_NOINL EPoint ed_lincomb(const u256 s, const u256 k, const EPoint negA, const uint32_t* btab) {
  constexpr int NR = 1 << (WR - 1);
  ENiels tab[NR];
  EPoint cur = negA;
  tab[0] = Edw::to_niels(cur);
  EPoint two = Edw::dbl(negA);
  cur = two;
  tab[1] = Edw::to_niels(cur);
#pragma unroll 1
  for (int i = 2; i < NR; ++i) {
    cur = Edw::add(cur, tab[0]);
    tab[i] = Edw::to_niels(cur);
  }
  // both scalars are < l < 2^253
  constexpr int JR = (254 + WR - 1) / WR;
  constexpr int JG = (254 + WG - 1) / WG;
  constexpr int TOP = ((JR - 1) * WR > (JG - 1) * WG) ? (JR - 1) * WR : (JG - 1) * WG;
  EPoint acc = Edw::identity();
#pragma unroll 1
  for (int pos = TOP; pos >= 0; --pos) {
    acc = Edw::dbl(acc, pos % WR == 0 || pos % WG == 0);
    // [k](-A)'s then [s]B's window through one addition site (one copy of the
    // addition in the loop: see k1_glv_lincomb)
    const uint32_t first = pos % WR == 0 ? 0u : 1u;
    const uint32_t last = pos % WG == 0 ? 2u : 1u;
#pragma unroll 1
    for (uint32_t src = first; src < last; ++src) {
      bool neg;
      const uint32_t d = src == 0 ? booth_digit(k, pos / WR, WR, neg) : booth_digit(s, pos / WG, WG, neg);
      if (!d) continue;
      ENiels e;
      if (src == 0) {
        e = tab[d - 1];
      } else {
        const EAffNiels g = load_eniels<WG>(btab, d - 1);
        e.ypx = g.ypx;
        e.ymx = g.ymx;
        e.z = u256_zero();  // unused: affine
        e.t2d = g.t2d;
      }
      if (neg) e = Edw::neg(e);
      // T only where a generator addition follows at this position; none after
      // the generator's (a doubling or the compression comes next)
      acc = Edw::add_either(acc, e, src == 1, src == 0 && pos % WG == 0);
    }
  }
  return acc;
}

// Verify one signature: A must decompress (as constructing a VerifyingKey
// does), S must be canonical (S < l, dalek without legacy_compatibility),
// and compress([S]B - [k]A) must equal the R bytes.  Follows
// src/wgsl/main/ed25519_eddsa_main.wgsl:23-113 and
// src/curve_algos/ed25519_eddsa.rs:49-77; adds the S < l check the reference
// GPU path lacks (src/wgsl/main/ed25519_eddsa_main_0.wgsl:45-54).
// challenge(R, A) returns k = SHA-512(R || A || M) mod l; it runs only after
// the key and S checks passed.
template <int WR = ED_WR, int WG = ED_WG, class Challenge>
SG_HD uint8_t ed25519_point_with(const uint32_t sig[16], const uint32_t pk[8], const uint32_t* btab, Challenge challenge, EPoint& Rp) {
  u256 aenc;
#pragma unroll
  for (int k = 0; k < 8; ++k) aenc.w[k] = pk[k];
  EPoint A;
  if (!Edw::decompress(aenc, A)) return ST_NO_POINT;
  u256 s, renc;
#pragma unroll
  for (int k = 0; k < 8; ++k) { renc.w[k] = sig[k]; s.w[k] = sig[8 + k]; }
  if (u256_gte(s, EdScalarC::N())) return ST_BAD_SCALAR;
  u256 k = challenge(renc, aenc);
  EPoint negA;
  negA.X = FpEd::neg(A.X);
  negA.Y = A.Y;
  negA.Z = A.Z;
  negA.T = FpEd::neg(A.T);
  Rp = ed_lincomb<WR, WG>(s, k, negA, btab);
  return ST_OK;
}

// ST_OK when the encoding of R' = (X : Y : Z), given Z^-1, equals the R bytes
SG_HD uint8_t ed25519_compare(const EPoint& Rp, const u256& zi, const uint32_t sig[16]) {
  u256 x = FpEd::canon(FpEd::mul(Rp.X, zi));
  u256 y = FpEd::canon(FpEd::mul(Rp.Y, zi));
  y.w[7] |= (x.w[0] & 1u) << 31;
  u256 renc;
#pragma unroll
  for (int k = 0; k < 8; ++k) renc.w[k] = sig[k];
  return u256_eq(y, renc) ? ST_OK : ST_MISMATCH;
}

template <class Challenge>
SG_HD uint8_t ed25519_verify_with(const uint32_t sig[16], const uint32_t pk[8], const uint32_t* btab, Challenge challenge) {
  EPoint Rp;
  const uint8_t st = ed25519_point_with(sig, pk, btab, challenge, Rp);
  if (st != ST_OK) return st;
  u256 enc = Edw::compress(Rp);
  u256 renc;
#pragma unroll
  for (int k = 0; k < 8; ++k) renc.w[k] = sig[k];
  return u256_eq(enc, renc) ? ST_OK : ST_MISMATCH;
}

// the reference's API: 32-byte (fuel) messages
SG_HD uint8_t ed25519_verify(const uint32_t sig[16], const uint32_t msg[8], const uint32_t pk[8], const uint32_t* btab) {
  return ed25519_verify_with(sig, pk, btab, [&](const u256&, const u256&) { return ed_challenge(sig, pk, msg); });
}

// the batched engine's form: R' = [S]B - [k]A before its compression (whose
// inversion the engine shares across items); ST_OK means "compare pending"
template <int WR = ED_WR, int WG = ED_WG>
SG_HD uint8_t ed25519_point(const uint32_t sig[16], const uint32_t msg[8], const uint32_t pk[8], const uint32_t* btab, EPoint& Rp) {
  return ed25519_point_with<WR, WG>(sig, pk, btab, [&](const u256&, const u256&) { return ed_challenge(sig, pk, msg); }, Rp);
}

// a message of any length (msg: len bytes, device memory on the GPU)
SG_HD uint8_t ed25519_verify_raw(const uint32_t sig[16], const uint8_t* msg, uint32_t len, const uint32_t pk[8], const uint32_t* btab) {
  return ed25519_verify_with(sig, pk, btab, [&](const u256& renc, const u256& aenc) {
    uint32_t h[16];
    sha512_ed_raw<>(renc, aenc, msg, len, h);
    return reduce512_mod_l(h);
  });
}

}  // namespace sg
