// Curve arithmetic.
//
// Weierstrass curves (secp256k1 a = 0, P-256 a = -3) in Jacobian coordinates
// with exact handling of the exceptional cases (P = Q, P = -Q, infinity), and
// ed25519 in extended twisted Edwards coordinates with the complete unified
// addition.  Replaces the reference's projective add-2007-bl / dbl-2007-bl
// (src/wgsl/secp256k1_curve.wgsl:26-111), RCB-2015 (src/wgsl/secp256r1_curve.wgsl:34-146)
// and add-2008-hwcd-3 / dbl-2008-hwcd (src/wgsl/ed25519_curve.wgsl:19-100).
//
// Scalar multiplication is Shamir-Strauss over signed fixed windows (Booth
// recoding): every window of every scalar contributes exactly one table
// addition at a fixed bit position, so all lanes of a warp follow the same
// control flow.  (The reference's double-and-add / wNAF-style loops branch
// per bit, src/wgsl/secp256k1_curve.wgsl:277-294, 336-383.)
#pragma once
#include "field.cuh"

namespace sg {

// ---------------------------------------------------------------------------
// Booth digits: scalar k = sum_j d_j 2^(w j), d_j in [-2^(w-1), 2^(w-1)]
//   d_j = bits[jw, jw+w) + bit(jw-1) - 2^w * bit(jw+w-1)
// ---------------------------------------------------------------------------
SG_HD uint32_t u256_bits(const u256& k, int pos, int cnt) {  // bits [pos, pos+cnt), cnt <= 32, pos may be < 0
  if (pos >= 256) return 0;
  uint32_t lo, hi;
  if (pos < 0) {
    // only used for pos = -1 (the bit below window 0): treat as 0
    uint32_t v = (k.w[0] << 1);
    return v & ((cnt == 32) ? 0xffffffffu : ((1u << cnt) - 1u));
  }
  int wi = pos >> 5, sh = pos & 31;
  lo = k.w[wi];
  hi = (wi + 1 < 8) ? k.w[wi + 1] : 0u;
  uint64_t v = ((uint64_t)hi << 32) | lo;
  v >>= sh;
  return (uint32_t)v & ((cnt == 32) ? 0xffffffffu : ((1u << cnt) - 1u));
}

// returns |d| and sets neg
SG_HD uint32_t booth_digit(const u256& k, int j, int w, bool& neg) {
  // w+1 bits starting at jw-1
  uint32_t b = u256_bits(k, j * w - 1, w + 1);  // bit 0 = bit(jw-1)
  uint32_t top = (b >> w) & 1u;
  uint32_t val = (b >> 1) + (b & 1u);  // c_j + bit(jw-1), with c_j = w bits
  // d = val - 2^w * top
  int32_t d = (int32_t)val - (int32_t)(top << w);
  neg = d < 0;
  return (uint32_t)(neg ? -d : d);
}

// ---------------------------------------------------------------------------
// Weierstrass, Jacobian (X/Z^2, Y/Z^3); Z == 0 is the point at infinity
// ---------------------------------------------------------------------------
struct JPoint {
  u256 X, Y, Z;
};
struct APoint {
  u256 x, y;
};

template <class F, bool A_M3>
struct Weier {
  SG_HD static JPoint infinity() { JPoint r; r.X = F::one(); r.Y = F::one(); r.Z = F::zero(); return r; }
  // Z is exactly zero (not merely p) for the point at infinity: infinity()
  // sets it, the exceptional cases return infinity(), and every other Z is a
  // product of nonzero factors
  SG_HD static bool is_inf(const JPoint& p) { return u256_is_zero(p.Z); }
  SG_HD static JPoint from_affine(const APoint& a) { JPoint r; r.X = a.x; r.Y = a.y; r.Z = F::one(); return r; }

  // 2p in the form of dbl-2004-hmv: (2Y)^2 gives 4 Y^2 and, squared and
  // halved, 8 Y^4, which saves the small multiples' additions.
  // a = -3: M = 3 (X - Z^2)(X + Z^2), 4M + 4S; a = 0: M = 3 X^2, 3M + 4S.
  SG_HD static JPoint dbl(const JPoint& p) {
    JPoint r;
    u256 M;
    if (A_M3) {
      const u256 zz = F::sqr(p.Z);
      M = F::mul(F::sub(p.X, zz), F::add(p.X, zz));
    } else {
      M = F::sqr(p.X);
    }
    M = F::add(F::add(M, M), M);
    const u256 y2 = F::add(p.Y, p.Y);
    r.Z = F::mul(y2, p.Z);
    const u256 y4 = F::sqr(y2);      // 4 Y^2
    const u256 S = F::mul(y4, p.X);  // 4 X Y^2
    const u256 y8 = F::half(F::sqr(y4));  // 8 Y^4
    r.X = F::sub(F::sqr(M), F::add(S, S));
    r.Y = F::sub(F::mul(F::sub(S, r.X), M), y8);
    return r;
  }

  // p + q with q affine (madd-2004-hmv, 8M + 3S: one more multiply than
  // madd-2007-bl but six fewer additions), exceptional cases exact
  SG_HD static JPoint madd(const JPoint& p, const APoint& q) {
    if (is_inf(p)) return from_affine(q);
    u256 Z1Z1 = F::sqr(p.Z);
    u256 U2 = F::mul(q.x, Z1Z1);
    u256 S2 = F::mul(q.y, F::mul(p.Z, Z1Z1));
    u256 H = F::sub(U2, p.X);
    u256 rr = F::sub(S2, p.Y);
    if (F::is_zero(H)) {
      if (F::is_zero(rr)) return dbl(from_affine(q));
      return infinity();
    }
    u256 HH = F::sqr(H);
    u256 HHH = F::mul(H, HH);
    u256 V = F::mul(p.X, HH);
    JPoint r;
    r.X = F::sub(F::sub(F::sqr(rr), HHH), F::add(V, V));
    r.Y = F::sub(F::mul(rr, F::sub(V, r.X)), F::mul(p.Y, HHH));
    r.Z = F::mul(p.Z, H);
    return r;
  }

  // p + q, both Jacobian (add-2007-bl, 11M + 5S), exceptional cases exact
  SG_HD static JPoint add(const JPoint& p, const JPoint& q) {
    if (is_inf(p)) return q;
    if (is_inf(q)) return p;
    u256 Z1Z1 = F::sqr(p.Z);
    u256 Z2Z2 = F::sqr(q.Z);
    u256 U1 = F::mul(p.X, Z2Z2);
    u256 U2 = F::mul(q.X, Z1Z1);
    u256 S1 = F::mul(p.Y, F::mul(q.Z, Z2Z2));
    u256 S2 = F::mul(q.Y, F::mul(p.Z, Z1Z1));
    u256 H = F::sub(U2, U1);
    u256 rr = F::sub(S2, S1);
    if (F::is_zero(H)) {
      if (F::is_zero(rr)) return dbl(p);
      return infinity();
    }
    rr = F::add(rr, rr);
    u256 H2 = F::add(H, H);
    u256 I = F::sqr(H2);
    u256 J = F::mul(H, I);
    u256 V = F::mul(U1, I);
    JPoint r;
    r.X = F::sub(F::sub(F::sqr(rr), J), F::add(V, V));
    u256 sj = F::mul(S1, J);
    r.Y = F::sub(F::mul(rr, F::sub(V, r.X)), F::add(sj, sj));
    u256 zz = F::add(p.Z, q.Z);
    r.Z = F::mul(F::sub(F::sub(F::sqr(zz), Z1Z1), Z2Z2), H);
    return r;
  }

  SG_HD static JPoint neg(const JPoint& p) { JPoint r = p; r.Y = F::neg(p.Y); return r; }
  SG_HD static APoint neg(const APoint& p) { APoint r = p; r.y = F::neg(p.y); return r; }

  // affine (field representation) of a non-infinity point
  SG_HD static APoint to_affine(const JPoint& p) {
    u256 zi = F::inv(p.Z);
    u256 zi2 = F::sqr(zi);
    APoint a;
    a.x = F::mul(p.X, zi2);
    a.y = F::mul(p.Y, F::mul(zi2, zi));
    return a;
  }
};

// ---------------------------------------------------------------------------
// ed25519, extended coordinates (X:Y:Z:T), x = X/Z, y = Y/Z, xy = T/Z
// ---------------------------------------------------------------------------
struct EPoint {
  u256 X, Y, Z, T;
};
// precomputed addend: (Y+X, Y-X, Z, 2d*T); Z = 1 for affine tables
struct ENiels {
  u256 ypx, ymx, z, t2d;
};
struct EAffNiels {
  u256 ypx, ymx, t2d;
};

struct Edw {
  using F = FpEd;
  SG_HD static EPoint identity() { EPoint r; r.X = F::zero(); r.Y = F::one(); r.Z = F::one(); r.T = F::zero(); return r; }

  // dbl-2008-hwcd with a = -1: 4M + 4S; with need_t false the T coordinate
  // is left stale (3M + 4S): only valid when the next operation is a doubling,
  // which never reads T
  SG_HD static EPoint dbl(const EPoint& p, bool need_t = true) {
    u256 A = F::sqr(p.X);
    u256 B = F::sqr(p.Y);
    u256 C = F::sqr(p.Z);
    C = F::add(C, C);
    u256 H = F::add(A, B);
    u256 xy = F::add(p.X, p.Y);
    u256 E = F::sub(H, F::sqr(xy));
    u256 G = F::sub(A, B);
    u256 Fv = F::add(C, G);
    EPoint r;
    r.X = F::mul(E, Fv);
    r.Y = F::mul(G, H);
    r.T = need_t ? F::mul(E, H) : p.T;
    r.Z = F::mul(Fv, G);
    return r;
  }

  // p + q for either form of q: projective Niels (8M, complete), or (affine
  // set) affine Niels held in the same struct with q.z unused, which skips the
  // Z1 Z2 product (7M).  With need_t false T is left stale (one M fewer), for
  // a result that only a doubling reads.  One formula for both lets a doubling
  // chain add through one site.
  SG_HD static EPoint add_either(const EPoint& p, const ENiels& q, bool affine, bool need_t) {
    u256 A = F::mul(F::sub(p.Y, p.X), q.ymx);
    u256 B = F::mul(F::add(p.Y, p.X), q.ypx);
    u256 C = F::mul(p.T, q.t2d);
    u256 D = affine ? p.Z : F::mul(p.Z, q.z);
    D = F::add(D, D);
    u256 E = F::sub(B, A), Fv = F::sub(D, C), G = F::add(D, C), H = F::add(B, A);
    EPoint r;
    r.X = F::mul(E, Fv);
    r.Y = F::mul(G, H);
    r.T = need_t ? F::mul(E, H) : p.T;
    r.Z = F::mul(Fv, G);
    return r;
  }

  // p + q, q in projective Niels form
  SG_HD static EPoint add(const EPoint& p, const ENiels& q, bool need_t = true) { return add_either(p, q, false, need_t); }

  SG_HD static ENiels to_niels(const EPoint& p) {
    ENiels n;
    n.ypx = F::add(p.Y, p.X);
    n.ymx = F::sub(p.Y, p.X);
    n.z = p.Z;
    n.t2d = F::mul(p.T, F::D2());
    return n;
  }
  SG_HD static ENiels neg(const ENiels& q) { ENiels r; r.ypx = q.ymx; r.ymx = q.ypx; r.z = q.z; r.t2d = F::neg(q.t2d); return r; }

  // canonical encoding: y little-endian, sign of x in bit 255
  // (src/wgsl/ed25519_curve.wgsl compress; curve25519-dalek EdwardsPoint::compress)
  SG_HD static u256 compress(const EPoint& p) {
    u256 zi = F::inv(p.Z);
    u256 x = F::canon(F::mul(p.X, zi));
    u256 y = F::canon(F::mul(p.Y, zi));
    y.w[7] |= (x.w[0] & 1u) << 31;
    return y;
  }

  // curve25519-dalek sqrt_ratio_i (src/curve_algos/ed25519_eddsa.rs:160-184);
  // the comparisons and the sign test use canonical values
  SG_HD static bool sqrt_ratio_i(const u256& u, const u256& v, u256& r_out) {
    u256 v3 = F::mul(F::sqr(v), v);
    u256 v7 = F::mul(F::sqr(v3), v);
    u256 r = F::mul(F::mul(u, v3), F::pow_p58(F::mul(u, v7)));
    const u256 check = F::canon(F::mul(v, F::sqr(r)));
    const u256 uc = F::canon(u);
    const u256 nu = F::canon(F::neg(uc));
    bool correct = u256_eq(check, uc);
    bool flipped = u256_eq(check, nu);
    bool flipped_i = u256_eq(check, F::canon(F::mul(nu, F::SQRT_M1())));
    u256 ri = F::mul(r, F::SQRT_M1());
    r = F::canon(u256_select(flipped || flipped_i, ri, r));
    r = u256_select((r.w[0] & 1u) != 0, F::canon(F::neg(r)), r);
    r_out = r;
    return correct || flipped;
  }

  // CompressedEdwardsY::decompress with dalek semantics: y taken mod p from the
  // low 255 bits, x = non-negative root negated when the sign bit is set
  SG_HD static bool decompress(const u256& enc, EPoint& out) {
    u256 y = enc;
    uint32_t sign = y.w[7] >> 31;
    y.w[7] &= 0x7fffffffu;
    y = F::canon(y);
    u256 yy = F::sqr(y);
    u256 u = F::sub(yy, F::one());
    u256 v = F::add(F::mul(yy, F::D()), F::one());
    u256 x;
    bool ok = sqrt_ratio_i(u, v, x);
    x = u256_select(sign != 0, F::neg(x), x);
    out.X = x;
    out.Y = y;
    out.Z = F::one();
    out.T = F::mul(x, y);
    return ok;
  }
};

}  // namespace sg
