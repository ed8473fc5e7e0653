// Generator tables, computed once on the host with the same field and curve
// code the kernels run.
//
//  * kernel tables: multiples 1..32768 of the generator (affine; Niels form for
//    ed25519) in the field representation the kernels use;
//  * the reference's table_limbs encoding: precompute::*_bases(log_limb_size)
//    (src/precompute.rs:14-69) = [1G .. 16G], each coordinate as
//    v * 2^(L * nl) mod p in nl little-endian L-bit limbs (x, y for the
//    Weierstrass curves, x, y, t = x*y for ed25519).
#pragma once
#include <algorithm>
#include <vector>

#include "recover.cuh"

namespace sg {

enum Curve : int { CURVE_SECP256K1 = 0, CURVE_SECP256R1 = 1, CURVE_ED25519 = 2 };

inline u256 k1_gx() { return SG_U256(0x16f81798u, 0x59f2815bu, 0x2dce28d9u, 0x029bfcdbu, 0xce870b07u, 0x55a06295u, 0xf9dcbbacu, 0x79be667eu); }
inline u256 k1_gy() { return SG_U256(0xfb10d4b8u, 0x9c47d08fu, 0xa6855419u, 0xfd17b448u, 0x0e1108a8u, 0x5da4fbfcu, 0x26a3c465u, 0x483ada77u); }
inline u256 r1_gx() { return SG_U256(0xd898c296u, 0xf4a13945u, 0x2deb33a0u, 0x77037d81u, 0x63a440f2u, 0xf8bce6e5u, 0xe12c4247u, 0x6b17d1f2u); }
inline u256 r1_gy() { return SG_U256(0x37bf51f5u, 0xcbb64068u, 0x6b315eceu, 0x2bce3357u, 0x7c0f9e16u, 0x8ee7eb4au, 0xfe1a7f9bu, 0x4fe342e2u); }
inline u256 ed_bx() { return SG_U256(0x8f25d51au, 0xc9562d60u, 0x9525a7b2u, 0x692cc760u, 0xfdd6dc5cu, 0xc0a4e231u, 0xcd6e53feu, 0x216936d3u); }
inline u256 ed_by() { return SG_U256(0x66666658u, 0x66666666u, 0x66666666u, 0x66666666u, 0x66666666u, 0x66666666u, 0x66666666u, 0x66666666u); }

// (i+1) * G for i < count, affine, in T::F's representation.  Jacobian
// multiples by mixed additions, made affine in chunks with one inversion each
// (Montgomery's simultaneous inversion).
template <class T>
inline void weier_multiples(const u256& gx, const u256& gy, int count, APoint* out) {
  using F = typename T::F;
  using W = Weier<F, T::A_M3>;
  constexpr int CHUNK = 256;
  APoint g;
  g.x = F::from_int(gx);
  g.y = F::from_int(gy);
  std::vector<JPoint> jp(CHUNK);
  std::vector<u256> pre(CHUNK);
  JPoint acc = W::from_affine(g);
  for (int base = 0; base < count; base += CHUNK) {
    const int m = std::min(CHUNK, count - base);
    for (int i = 0; i < m; ++i) {
      jp[i] = acc;
      acc = W::madd(acc, g);  // (i+1) G is never the point at infinity
    }
    pre[0] = jp[0].Z;
    for (int i = 1; i < m; ++i) pre[i] = F::mul(pre[i - 1], jp[i].Z);
    u256 inv = F::inv(pre[m - 1]);
    for (int i = m - 1; i >= 0; --i) {
      u256 zi = inv;
      if (i > 0) {
        zi = F::mul(inv, pre[i - 1]);
        inv = F::mul(inv, jp[i].Z);
      }
      const u256 z2 = F::sqr(zi);
      out[base + i].x = F::canon(F::mul(jp[i].X, z2));
      out[base + i].y = F::canon(F::mul(jp[i].Y, F::mul(z2, zi)));
    }
  }
}

// (i+1) * B for i < count, affine (x, y) as integers; chunked simultaneous
// inversion as above
inline void ed_multiples(int count, u256* xs, u256* ys) {
  using F = FpEd;
  constexpr int CHUNK = 256;
  EPoint b;
  b.X = ed_bx();
  b.Y = ed_by();
  b.Z = F::one();
  b.T = F::mul(b.X, b.Y);
  const ENiels bn = Edw::to_niels(b);
  std::vector<EPoint> ep(CHUNK);
  std::vector<u256> pre(CHUNK);
  EPoint acc = b;
  for (int base = 0; base < count; base += CHUNK) {
    const int m = std::min(CHUNK, count - base);
    for (int i = 0; i < m; ++i) {
      ep[i] = acc;
      acc = Edw::add(acc, bn);
    }
    pre[0] = ep[0].Z;
    for (int i = 1; i < m; ++i) pre[i] = F::mul(pre[i - 1], ep[i].Z);
    u256 inv = F::inv(pre[m - 1]);
    for (int i = m - 1; i >= 0; --i) {
      u256 zi = inv;
      if (i > 0) {
        zi = F::mul(inv, pre[i - 1]);
        inv = F::mul(inv, ep[i].Z);
      }
      xs[base + i] = F::canon(F::mul(ep[i].X, zi));
      ys[base + i] = F::canon(F::mul(ep[i].Y, zi));
    }
  }
}

// kernel table for the Weierstrass curves: `count` entries of 16 words (x, y)
template <class T>
inline void build_weier_gtab(const u256& gx, const u256& gy, uint32_t* out, int count = ECDSA_GTAB) {
  std::vector<APoint> pts(count);
  weier_multiples<T>(gx, gy, count, pts.data());
  for (int i = 0; i < count; ++i)
    for (int k = 0; k < 8; ++k) {
      out[i * 16 + k] = pts[i].x.w[k];
      out[i * 16 + 8 + k] = pts[i].y.w[k];
    }
}

// secp256k1 GLV table: multiples 1..count of G, then the same multiples of 2^128 G
inline void build_k1_glv_gtab(uint32_t* out, int count = ECDSA_GTAB) {
  using F = FpK1;
  using W = Weier<F, false>;
  build_weier_gtab<K1Traits>(k1_gx(), k1_gy(), out, count);
  APoint g;
  g.x = k1_gx();
  g.y = k1_gy();
  JPoint h = W::from_affine(g);
  for (int i = 0; i < 128; ++i) h = W::dbl(h);
  APoint ha = W::to_affine(h);
  build_weier_gtab<K1Traits>(F::to_int(ha.x), F::to_int(ha.y), out + (size_t)count * 16, count);
}

// kernel table for ed25519: `count` entries of 24 words (y+x, y-x, 2d*x*y)
inline void build_ed_btab(uint32_t* out, int count = ED_GTAB) {
  std::vector<u256> xs(count), ys(count);
  ed_multiples(count, xs.data(), ys.data());
  for (int i = 0; i < count; ++i) {
    u256 ypx = FpEd::canon(FpEd::add(ys[i], xs[i]));
    u256 ymx = FpEd::canon(FpEd::sub(ys[i], xs[i]));
    u256 t2d = FpEd::canon(FpEd::mul(FpEd::mul(xs[i], ys[i]), FpEd::D2()));
    for (int k = 0; k < 8; ++k) {
      out[i * 24 + k] = ypx.w[k];
      out[i * 24 + 8 + k] = ymx.w[k];
      out[i * 24 + 16 + k] = t2d.w[k];
    }
  }
}

// The kernels' generator tables, built once per process (thread-safe static
// initialisation): secp256k1 (G and 2^128 G multiples), P-256, ed25519; for
// 16-bit windows (tab, read from global memory) and 8-bit windows (small,
// staged into shared memory)
struct KernelTables {
  std::vector<uint32_t> tab[3];
  std::vector<uint32_t> small[3];
};
inline const KernelTables& kernel_tables() {
  static const KernelTables t = [] {
    KernelTables k;
    k.tab[CURVE_SECP256K1].resize(2 * ECDSA_GTAB * 16);
    k.tab[CURVE_SECP256R1].resize(ECDSA_GTAB * 16);
    k.tab[CURVE_ED25519].resize(ED_GTAB * 24);
    build_k1_glv_gtab(k.tab[CURVE_SECP256K1].data());
    build_weier_gtab<R1Traits>(r1_gx(), r1_gy(), k.tab[CURVE_SECP256R1].data());
    build_ed_btab(k.tab[CURVE_ED25519].data());
    k.small[CURVE_SECP256K1].resize(2 * SMALL_GTAB * 16);
    k.small[CURVE_SECP256R1].resize(SMALL_GTAB * 16);
    k.small[CURVE_ED25519].resize(SMALL_GTAB * 24);
    build_k1_glv_gtab(k.small[CURVE_SECP256K1].data(), SMALL_GTAB);
    build_weier_gtab<R1Traits>(r1_gx(), r1_gy(), k.small[CURVE_SECP256R1].data(), SMALL_GTAB);
    build_ed_btab(k.small[CURVE_ED25519].data(), SMALL_GTAB);
    return k;
  }();
  return t;
}

// ---------------------------------------------------------------------------
// reference table_limbs encoding
// ---------------------------------------------------------------------------
constexpr int BASES_COUNT = 16;                       // 2^WINDOW_SIZE, src/precompute.rs:12
constexpr uint32_t MIN_LOG_LIMB = 11, MAX_LOG_LIMB = 15;  // src/wgsl/mont.wgsl:12,37

inline int bases_num_limbs(uint32_t L) { return (int)((256 + L - 1) / L); }

inline int bases_len(int curve, uint32_t L) {
  int coords = curve == CURVE_ED25519 ? 3 : 2;
  return BASES_COUNT * coords * bases_num_limbs(L);
}

// v (integer < 2^256) into nl limbs of L bits
inline void split_limbs(const u256& v, uint32_t L, uint32_t* out) {
  int nl = bases_num_limbs(L);
  for (int i = 0; i < nl; ++i) {
    uint32_t bit = (uint32_t)i * L, acc = 0;
    for (uint32_t b = 0; b < L; ++b) {
      uint32_t pos = bit + b;
      if (pos < 256) acc |= ((v.w[pos >> 5] >> (pos & 31)) & 1u) << b;
    }
    out[i] = acc;
  }
}

// 2^e mod m by repeated doubling (m > 2^255 or the ed25519 prime)
inline u256 pow2_mod(uint32_t e, const u256& m) {
  u256 v = u256_small(1);
  for (uint32_t i = 0; i < e; ++i) v = mod_add(v, v, m);
  return v;
}

// integer product mod p through the curve's field
template <class F>
inline u256 int_mulmod(const u256& a, const u256& b) {
  return F::to_int(F::mul(F::from_int(a), F::from_int(b)));
}

// fills out[bases_len(curve, L)]; returns the length, or -1 for an unsupported L
inline int build_bases(int curve, uint32_t L, uint32_t* out) {
  if (L < MIN_LOG_LIMB || L > MAX_LOG_LIMB) return -1;
  const int nl = bases_num_limbs(L);
  const uint32_t e = (uint32_t)nl * L;
  if (curve == CURVE_SECP256K1 || curve == CURVE_SECP256R1) {
    APoint pts[BASES_COUNT];
    u256 xs[BASES_COUNT], ys[BASES_COUNT], rl;
    if (curve == CURVE_SECP256K1) {
      weier_multiples<K1Traits>(k1_gx(), k1_gy(), BASES_COUNT, pts);
      rl = pow2_mod(e, FpK1::P());
      for (int i = 0; i < BASES_COUNT; ++i) {
        xs[i] = int_mulmod<FpK1>(FpK1::to_int(pts[i].x), rl);
        ys[i] = int_mulmod<FpK1>(FpK1::to_int(pts[i].y), rl);
      }
    } else {
      weier_multiples<R1Traits>(r1_gx(), r1_gy(), BASES_COUNT, pts);
      rl = pow2_mod(e, FpR1::P());
      for (int i = 0; i < BASES_COUNT; ++i) {
        xs[i] = int_mulmod<FpR1>(FpR1::to_int(pts[i].x), rl);
        ys[i] = int_mulmod<FpR1>(FpR1::to_int(pts[i].y), rl);
      }
    }
    for (int i = 0; i < BASES_COUNT; ++i) {
      split_limbs(xs[i], L, out + (2 * i) * nl);
      split_limbs(ys[i], L, out + (2 * i + 1) * nl);
    }
    return bases_len(curve, L);
  }
  if (curve == CURVE_ED25519) {
    u256 xs[BASES_COUNT], ys[BASES_COUNT];
    ed_multiples(BASES_COUNT, xs, ys);
    u256 rl = pow2_mod(e, FpEd::P());
    for (int i = 0; i < BASES_COUNT; ++i) {
      u256 t = FpEd::mul(xs[i], ys[i]);
      split_limbs(FpEd::canon(FpEd::mul(xs[i], rl)), L, out + (3 * i) * nl);
      split_limbs(FpEd::canon(FpEd::mul(ys[i], rl)), L, out + (3 * i + 1) * nl);
      split_limbs(FpEd::canon(FpEd::mul(t, rl)), L, out + (3 * i + 2) * nl);
    }
    return bases_len(curve, L);
  }
  return -1;
}

}  // namespace sg
