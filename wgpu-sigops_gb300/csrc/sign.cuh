// Signing, for generating synthetic workloads on the device (benchmarks and
// large tests).  Not on the reference's path: the reference signs on the CPU
// with fuel-crypto / p256 / ed25519-dalek in its tests
// (src/tests/secp256k1_ecdsa.rs:30-36, src/tests/ed25519_eddsa.rs:22-24).
// Produces the same encodings those crates produce: low-s ECDSA with the y
// parity in bit 7 of byte 32 (fuel), RFC 8032 Ed25519.
#pragma once
#include "recover.cuh"

namespace sg {

// ECDSA with secret d and nonce k (both 32 bytes big-endian).  Returns 0, or
// 1 when (d, k) cannot sign (k or d outside [1, n-1], r = 0, R.x >= n, s = 0).
template <class T>
SG_HD uint8_t ecdsa_sign(const uint32_t d_w[8], const uint32_t k_w[8], const uint32_t msg[8], const uint32_t* gtab, uint32_t sig[16],
                         uint32_t pub[16]) {
  using F = typename T::F;
  using S = typename T::S;
  using W = Weier<F, T::A_M3>;
  const u256 N = S::N();
  u256 d = be_words_to_u256(d_w), k = be_words_to_u256(k_w);
  u256 z = reduce_once(be_words_to_u256(msg), N);
  if (u256_is_zero(d) || u256_gte(d, N) || u256_is_zero(k) || u256_gte(k, N)) return 1;
  APoint g = load_apoint(gtab, 0);
  JPoint Rj = ecdsa_lincomb<T>(k, u256_zero(), g, gtab);
  APoint R = W::to_affine(Rj);
  u256 rx = F::to_int(R.x);
  uint32_t parity = F::to_int(R.y).w[0] & 1u;
  if (u256_is_zero(rx) || u256_gte(rx, N)) return 1;
  u256 kinv_m = S::from_int(S::inv_int(k));
  u256 t = S::add(z, S::mul(rx, S::from_int(d)));
  u256 s = S::mul(t, kinv_m);
  if (u256_is_zero(s)) return 1;
  u256 ns;
  u256_sub(ns, N, s);
  if (u256_gte(s, ns)) {  // s > n/2 (n odd): use n - s and flip the parity
    s = ns;
    parity ^= 1u;
  }
  u256_to_be_words(rx, sig);
  u256_to_be_words(s, sig + 8);
  sig[8] |= parity << 7;
  APoint Q = W::to_affine(ecdsa_lincomb<T>(d, u256_zero(), g, gtab));
  u256_to_be_words(F::to_int(Q.x), pub);
  u256_to_be_words(F::to_int(Q.y), pub + 8);
  return 0;
}

// RFC 8032 Ed25519 signature of a 32-byte message under a 32-byte seed
SG_HD void ed25519_sign(const uint32_t seed[8], const uint32_t msg[8], const uint32_t* btab, uint32_t sig[16], uint32_t pk[8]) {
  uint32_t h[16], buf[24], hr[16];
  sha512_fixed<32>(seed, h);
  h[0] &= 0xfffffff8u;  // clamp: clear bits 0..2, clear bit 255, set bit 254
  h[7] &= 0x7fffffffu;
  h[7] |= 0x40000000u;
  u256 a;
#pragma unroll
  for (int i = 0; i < 8; ++i) a.w[i] = h[i];
  u256 a_l = ScEd::to_int(ScEd::from_int(a));  // a mod l: a * B = (a mod l) * B
  EPoint id = Edw::identity();
  u256 A = Edw::compress(ed_lincomb(a_l, u256_zero(), id, btab));
#pragma unroll
  for (int i = 0; i < 8; ++i) { buf[i] = h[8 + i]; buf[8 + i] = msg[i]; }
  sha512_fixed<64>(buf, hr);
  u256 r = reduce512_mod_l(hr);
  u256 R = Edw::compress(ed_lincomb(r, u256_zero(), id, btab));
#pragma unroll
  for (int i = 0; i < 8; ++i) { sig[i] = R.w[i]; pk[i] = A.w[i]; }
  u256 k = ed_challenge(sig, pk, msg);
  u256 S = ScEd::add(r, ScEd::mul(k, ScEd::from_int(a)));
#pragma unroll
  for (int i = 0; i < 8; ++i) sig[8 + i] = S.w[i];
}

}  // namespace sg
