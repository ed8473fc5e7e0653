// One-block SHA-512: the 96-byte ed25519 challenge preimage R || A || M, and
// the 32- and 64-byte inputs of RFC 8032 signing (workload generation).
//
// Replaces src/wgsl/sha512.wgsl:1-194 (`sha512_96`, 64-bit words emulated as
// vec2<u32>); here 64-bit words are native and the 80 rounds are unrolled with
// the round constants as immediates.  The message schedule is built in place
// for the fixed 96-byte length (padding byte at offset 96, bit length 768).
// Constants: FIPS 180-4 section 4.2.3 / 5.3.5.
#pragma once
#include "arith.cuh"

namespace sg {

SG_HD uint64_t rotr64(uint64_t x, int n) { return (x >> n) | (x << (64 - n)); }

// One-block SHA-512 of NB bytes (NB a multiple of 8, at most 104).
// m: the input bytes as NB/4 little-endian u32 words (as loaded from memory).
// out: the 64-byte digest as 16 little-endian u32 words (digest byte order).
SG_HD void sha512_init(uint64_t st[8]) {
  st[0] = 0x6a09e667f3bcc908ull;
  st[1] = 0xbb67ae8584caa73bull;
  st[2] = 0x3c6ef372fe94f82bull;
  st[3] = 0xa54ff53a5f1d36f1ull;
  st[4] = 0x510e527fade682d1ull;
  st[5] = 0x9b05688c2b3e6c1full;
  st[6] = 0x1f83d9abfb41bd6bull;
  st[7] = 0x5be0cd19137e2179ull;
}

// one 128-byte block (w: 16 big-endian 64-bit words, overwritten) into st
SG_HD void sha512_compress(uint64_t st[8], uint64_t w[16]) {
  const uint64_t K[80] = {
    0x428a2f98d728ae22ull, 0x7137449123ef65cdull, 0xb5c0fbcfec4d3b2full, 0xe9b5dba58189dbbcull,
    0x3956c25bf348b538ull, 0x59f111f1b605d019ull, 0x923f82a4af194f9bull, 0xab1c5ed5da6d8118ull,
    0xd807aa98a3030242ull, 0x12835b0145706fbeull, 0x243185be4ee4b28cull, 0x550c7dc3d5ffb4e2ull,
    0x72be5d74f27b896full, 0x80deb1fe3b1696b1ull, 0x9bdc06a725c71235ull, 0xc19bf174cf692694ull,
    0xe49b69c19ef14ad2ull, 0xefbe4786384f25e3ull, 0x0fc19dc68b8cd5b5ull, 0x240ca1cc77ac9c65ull,
    0x2de92c6f592b0275ull, 0x4a7484aa6ea6e483ull, 0x5cb0a9dcbd41fbd4ull, 0x76f988da831153b5ull,
    0x983e5152ee66dfabull, 0xa831c66d2db43210ull, 0xb00327c898fb213full, 0xbf597fc7beef0ee4ull,
    0xc6e00bf33da88fc2ull, 0xd5a79147930aa725ull, 0x06ca6351e003826full, 0x142929670a0e6e70ull,
    0x27b70a8546d22ffcull, 0x2e1b21385c26c926ull, 0x4d2c6dfc5ac42aedull, 0x53380d139d95b3dfull,
    0x650a73548baf63deull, 0x766a0abb3c77b2a8ull, 0x81c2c92e47edaee6ull, 0x92722c851482353bull,
    0xa2bfe8a14cf10364ull, 0xa81a664bbc423001ull, 0xc24b8b70d0f89791ull, 0xc76c51a30654be30ull,
    0xd192e819d6ef5218ull, 0xd69906245565a910ull, 0xf40e35855771202aull, 0x106aa07032bbd1b8ull,
    0x19a4c116b8d2d0c8ull, 0x1e376c085141ab53ull, 0x2748774cdf8eeb99ull, 0x34b0bcb5e19b48a8ull,
    0x391c0cb3c5c95a63ull, 0x4ed8aa4ae3418acbull, 0x5b9cca4f7763e373ull, 0x682e6ff3d6b2b8a3ull,
    0x748f82ee5defb2fcull, 0x78a5636f43172f60ull, 0x84c87814a1f0ab72ull, 0x8cc702081a6439ecull,
    0x90befffa23631e28ull, 0xa4506cebde82bde9ull, 0xbef9a3f7b2c67915ull, 0xc67178f2e372532bull,
    0xca273eceea26619cull, 0xd186b8c721c0c207ull, 0xeada7dd6cde0eb1eull, 0xf57d4f7fee6ed178ull,
    0x06f067aa72176fbaull, 0x0a637dc5a2c898a6ull, 0x113f9804bef90daeull, 0x1b710b35131c471bull,
    0x28db77f523047d84ull, 0x32caab7b40c72493ull, 0x3c9ebe0a15c9bebcull, 0x431d67c49c100d4cull,
    0x4cc5d4becb3e42b6ull, 0x597f299cfc657e2aull, 0x5fcb6fab3ad6faecull, 0x6c44198c4a475817ull,
  };
  uint64_t a = st[0], b = st[1], c = st[2], d = st[3], e = st[4], f = st[5], g = st[6], h = st[7];
#pragma unroll
  for (int i = 0; i < 80; ++i) {
    uint64_t wi;
    if (i < 16) {
      wi = w[i];
    } else {
      uint64_t w15 = w[(i - 15) & 15], w2 = w[(i - 2) & 15];
      uint64_t s0 = rotr64(w15, 1) ^ rotr64(w15, 8) ^ (w15 >> 7);
      uint64_t s1 = rotr64(w2, 19) ^ rotr64(w2, 61) ^ (w2 >> 6);
      wi = w[i & 15] + s0 + w[(i - 7) & 15] + s1;
      w[i & 15] = wi;
    }
    uint64_t S1 = rotr64(e, 14) ^ rotr64(e, 18) ^ rotr64(e, 41);
    uint64_t ch = (e & f) ^ (~e & g);
    uint64_t t1 = h + S1 + ch + K[i] + wi;
    uint64_t S0 = rotr64(a, 28) ^ rotr64(a, 34) ^ rotr64(a, 39);
    uint64_t maj = (a & b) ^ (a & c) ^ (b & c);
    uint64_t t2 = S0 + maj;
    h = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
  }
  st[0] += a;
  st[1] += b;
  st[2] += c;
  st[3] += d;
  st[4] += e;
  st[5] += f;
  st[6] += g;
  st[7] += h;
}

// the 64-byte digest as 16 little-endian u32 words (digest byte order)
SG_HD void sha512_digest(const uint64_t st[8], uint32_t out[16]) {
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    out[2 * i] = bswap32((uint32_t)(st[i] >> 32));
    out[2 * i + 1] = bswap32((uint32_t)st[i]);
  }
}

// One-block SHA-512 of NB bytes (NB a multiple of 8, at most 104).
// m: the input bytes as NB/4 little-endian u32 words (as loaded from memory).
// out: the 64-byte digest as 16 little-endian u32 words (digest byte order).
template <int NB>
SG_HD void sha512_fixed(const uint32_t* m, uint32_t out[16]) {
  static_assert(NB % 8 == 0 && NB <= 104, "one-block input");
  uint64_t w[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    if (i < NB / 8) {
      w[i] = ((uint64_t)bswap32(m[2 * i]) << 32) | bswap32(m[2 * i + 1]);
    } else if (i == NB / 8) {
      w[i] = 0x8000000000000000ull;
    } else {
      w[i] = 0;
    }
  }
  w[15] = (uint64_t)NB * 8;
  uint64_t st[8];
  sha512_init(st);
  sha512_compress(st, w);
  sha512_digest(st, out);
}

// the ed25519 challenge preimage R || A || M
SG_HD void sha512_96(const uint32_t m[24], uint32_t out[16]) { sha512_fixed<96>(m, out); }

// SHA-512 of R || A || msg for a message of any length (ed25519 over raw
// messages): R and A as 8 little-endian u32 words each, msg as bytes (device
// memory on the GPU).  ceil((64 + len + 17) / 128) blocks; every lane of a
// warp runs the block count of its own message.
template <int = 0>
SG_NOINL void sha512_ed_raw(const u256 R, const u256 A, const uint8_t* msg, uint32_t len, uint32_t out[16]) {
  const uint64_t total = 64ull + len;
  const uint64_t nblocks = (total + 17 + 127) / 128;
  uint64_t st[8];
  sha512_init(st);
#pragma unroll 1
  for (uint64_t blk = 0; blk < nblocks; ++blk) {
    uint64_t w[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const uint64_t base = blk * 128 + (uint64_t)t * 8;
      uint64_t v = 0;
      if (base + 8 <= 64) {  // a whole word of R || A
        const uint32_t* src = base < 32 ? R.w : A.w;
        const int k = (int)((base & 31) >> 2);
        v = ((uint64_t)bswap32(src[k]) << 32) | bswap32(src[k + 1]);
      } else {
#pragma unroll 1
        for (int q = 0; q < 8; ++q) {
          const uint64_t pos = base + q;
          uint32_t byte = 0;
          if (pos < 64) {
            const uint32_t* src = pos < 32 ? R.w : A.w;
            byte = (src[(pos & 31) >> 2] >> (8 * (pos & 3))) & 0xffu;
          } else if (pos < total) {
            byte = msg[pos - 64];
          } else if (pos == total) {
            byte = 0x80u;
          }
          v = (v << 8) | byte;
        }
      }
      w[t] = v;
    }
    if (blk + 1 == nblocks) {  // 128-bit big-endian bit length in the last 16 bytes
      w[14] = 0;
      w[15] = total * 8;
    }
    sha512_compress(st, w);
  }
  sha512_digest(st, out);
}

}  // namespace sg
