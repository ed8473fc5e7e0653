// Threads per signature, measured: secp256k1 recovery by one thread per
// signature (the plain path) or by a pair of lanes per signature.
//
// In SIMT a warp issues one instruction stream for its 32 lanes, so splitting
// a signature over lanes shortens it only where the lanes run the same
// instructions on different data.  secp256k1's GLV decomposition gives such a
// split: u2 R = k1 R + k2 phi(R) and u1 G = a G + b 2^128 G, so the even lane
// of a pair adds k1's and a's window entries and the odd lane k2's and b's,
// each over its own copy of the doubling chain, and the pair combines the two
// partial sums with one addition.  Everything else (decoding, the square
// root, r^-1, the table of multiples of R, the final inversion) both lanes
// run on the same data.  A signature then takes the doubling chain plus half
// the window additions plus one addition, instead of the chain plus all the
// additions; it costs two lanes.  P-256 and ed25519 have no such endomorphism:
// splitting their windows between lanes makes the lanes branch differently at
// every window, which a warp runs one after the other.
//
// The plain secp256k1 path uses the pair for batches that leave most lanes of
// the GPU idle (launch_plain_k1_small); sigops_probe_k1_lanes measures both
// forms.  Results are checked equal to the plain kernel's.
#include "plain.cuh"

namespace sg {

// half 0: k1 R + a G; half 1: k2 phi(R) + b 2^128 G (same instruction stream)
template <int WR = ECDSA_WR, int WG = ECDSA_WG>
SG_NOINL JPoint k1_glv_half(const u256 u1, const u256 u2, const APoint R, const uint32_t* gtab2, uint32_t half) {
  using F = FpK1;
  using W = Weier<F, false>;
  constexpr int NR = 1 << (WR - 1);
  constexpr int HALF = 1 << (WG - 1);
  u256 k1, k2;
  bool neg1, neg2;
  K1Glv::split(u2, k1, neg1, k2, neg2);
  APoint R1 = neg1 ? W::neg(R) : R;
  APoint tab[NR];
  u256 zc;  // the chain runs on E' (coz_table_iso); generator entries enter as psi(P)
  coz_table_iso<F, NR>(R1, tab, zc);
  const u256 zc2 = F::sqr(zc);
  const u256 zc3 = F::mul(zc2, zc);
  const bool flip = half ? neg1 != neg2 : false;
  const u256 beta = K1Glv::BETA();
  u256 a = u1, b = u256_zero();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    b.w[k] = u1.w[4 + k];
    a.w[4 + k] = 0;
  }
  const u256 kr = half ? k2 : k1;
  const u256 kg = half ? b : a;
  const uint32_t goff = half ? (uint32_t)HALF : 0u;
  constexpr int JR = (130 + WR - 1) / WR;
  constexpr int JG = (129 + WG - 1) / WG;
  constexpr int TOP = ((JR - 1) * WR > (JG - 1) * WG) ? (JR - 1) * WR : (JG - 1) * WG;
  JPoint acc = W::infinity();
#pragma unroll 1
  for (int pos = TOP; pos >= 0; --pos) {
    acc = W::dbl(acc);
    // the R-side then the G-side window through one addition site
    const uint32_t first = pos % WR == 0 ? 0u : 1u;
    const uint32_t last = pos % WG == 0 ? 2u : 1u;
#pragma unroll 1
    for (uint32_t src = first; src < last; ++src) {
      bool ng;
      const uint32_t d = src == 0 ? booth_digit(kr, pos / WR, WR, ng) : booth_digit(kg, pos / WG, WG, ng);
      if (!d) continue;
      APoint e;
      if (src == 0) {
        e = tab[d - 1];
        if (half) e.x = F::mul(e.x, beta);
        if (flip) ng = !ng;
      } else {
        e = iso_point<F>(load_apoint<WG>(gtab2, goff + d - 1), zc2, zc3);
      }
      if (ng) e = W::neg(e);
      acc = W::madd(acc, e);
    }
  }
  if (!W::is_inf(acc)) acc.Z = F::mul(acc.Z, zc);  // back to E; infinity keeps Z exactly 0
  return acc;
}

__device__ __forceinline__ u256 shfl_xor_u256(const u256& v, int m) {
  u256 r;
#pragma unroll
  for (int k = 0; k < 8; ++k) r.w[k] = __shfl_xor_sync(0xffffffffu, v.w[k], m);
  return r;
}

// One signature on the lane pair (lane, lane ^ 1); every lane of the warp
// takes part (a lane without an item works on a stand-in signature), since the
// pair exchanges its partial sums by shuffles
__device__ uint8_t k1_recover_pair(const uint32_t sig[16], const uint32_t msg[8], bool valid_in, const uint32_t* gtab, uint32_t out[16],
                                   uint32_t half) {
  using T = K1Traits;
  using F = FpK1;
  using S = typename T::S;
  using W = Weier<F, false>;
#pragma unroll
  for (int k = 0; k < 16; ++k) out[k] = 0;
  u256 r, s, z;
  APoint R;
  uint8_t st = valid_in ? ecdsa_prepare<T>(sig, msg, r, s, z, R) : (uint8_t)ST_BAD_SCALAR;
  if (st != ST_OK) {  // stand-in: u1 = u2 = 1 and R = G keep the lane on the common path
    r = u256_small(1);
    s = u256_small(1);
    z = u256_zero();
    const APoint g = load_apoint<ECDSA_WG>(gtab, 0);
    R = g;
  }
  const u256 rinv_m = S::from_int(S::inv_int(r));
  const u256 u2 = S::mul(s, rinv_m);
  const u256 u1 = S::neg(S::mul(z, rinv_m));
  JPoint acc = k1_glv_half(u1, u2, R, gtab, half);
  JPoint other;
  other.X = shfl_xor_u256(acc.X, 1);
  other.Y = shfl_xor_u256(acc.Y, 1);
  other.Z = shfl_xor_u256(acc.Z, 1);
  if (st != ST_OK) return st;
  JPoint Q;
  if (W::is_inf(acc)) Q = other;
  else if (W::is_inf(other)) Q = acc;
  else Q = half ? W::add(other, acc) : W::add(acc, other);
  if (W::is_inf(Q)) return ST_INFINITY;
  const APoint a = W::to_affine(Q);
  u256_to_be_words(F::to_int(a.x), out);
  u256_to_be_words(F::to_int(a.y), out + 8);
  return ST_OK;
}

template <int LANES>
__global__ void __launch_bounds__(256, 1) k1_lanes_kernel(const uint8_t* __restrict__ sigs, const uint8_t* __restrict__ msgs, size_t n,
                                                        const uint32_t* __restrict__ gtab, uint8_t* __restrict__ out,
                                                        uint8_t* __restrict__ status) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t s[16], m[8], o[16];
  if constexpr (LANES == 1) {
    if (t >= n) return;
    load_words(sigs, t, 16, s);
    load_words(msgs, t, 8, m);
    const uint8_t st = ecdsa_recover<K1Traits, true>(s, m, gtab, o);
    store_words(out, t, 16, o);
    status[t] = st;
  } else {
    const size_t i = t >> 1;
    const uint32_t half = (uint32_t)(t & 1u);
    const bool in = i < n;
    if (in) {
      load_words(sigs, i, 16, s);
      load_words(msgs, i, 8, m);
    } else {
#pragma unroll
      for (int k = 0; k < 16; ++k) s[k] = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) m[k] = 0;
    }
    const uint8_t st = k1_recover_pair(s, m, in, gtab, o, half);
    if (in && half == 0) {
      store_words(out, i, 16, o);
      status[i] = st;
    }
  }
}

// lanes 1 or 2 per signature; block: threads per block (a multiple of 32 up
// to 256; 0 = 256, or fewer for a batch smaller than one block)
cudaError_t launch_k1_lanes(int lanes, const uint8_t* sigs, const uint8_t* msgs, size_t n, int block_req, const uint32_t* gtab,
                            uint8_t* out, uint8_t* status, cudaStream_t stream) {
  const size_t tot = (size_t)lanes * n;
  unsigned block = block_req > 0 ? (unsigned)block_req : 256u;
  if (block > 256u || block % 32u) return cudaErrorInvalidValue;
  if (tot < block) block = (unsigned)((tot + 31) / 32 * 32);
  const unsigned grid = (unsigned)((tot + block - 1) / block);
  if (lanes == 1) k1_lanes_kernel<1><<<grid, block, 0, stream>>>(sigs, msgs, n, gtab, out, status);
  else k1_lanes_kernel<2><<<grid, block, 0, stream>>>(sigs, msgs, n, gtab, out, status);
  return cudaGetLastError();
}

// Warp phases, measured: secp256k1 recovery, one thread per signature, by
// persistent warps that each take 32 items at a time.  Free-running (SYNC
// false), a warp takes its next items as soon as it is done, as the serving
// kernel's warps do, and after a few groups the warps of an SM are spread over
// the phases of a recovery (square root, inversions, doubling chain) at any
// one time.  Synchronised (SYNC true), a block's warps start every group
// together, as a plain kernel's block does.  The two differ in how much of the
// code the warps of an SM need at once, so in how often a warp waits for its
// next instruction to be fetched.  times[2g], times[2g + 1]: global-timer
// start and end of group g (items 32g .. 32g + 31).
__device__ __forceinline__ unsigned long long phase_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <bool SYNC>
__global__ void __launch_bounds__(256, 1) k1_phase_kernel(const uint8_t* __restrict__ sigs, const uint8_t* __restrict__ msgs, size_t n,
                                                          const uint32_t* __restrict__ gtab, uint8_t* __restrict__ out,
                                                          uint8_t* __restrict__ status, unsigned long long* counter, unsigned long long* times) {
  __shared__ unsigned long long block_base;
  const unsigned lane = threadIdx.x & 31u;
#pragma unroll 1
  for (;;) {
    unsigned long long base = 0;
    if constexpr (SYNC) {
      __syncthreads();  // every warp is done reading block_base
      if (threadIdx.x == 0) block_base = atomicAdd(counter, (unsigned long long)blockDim.x);
      __syncthreads();
      if (block_base >= n) return;  // the same for the whole block
      base = block_base + 32ull * (threadIdx.x >> 5);
    } else {
      if (lane == 0) base = atomicAdd(counter, 32ull);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= n) return;
    }
    if (base < n) {  // a synchronised block's last round may leave warps without items
      const unsigned long long t0 = phase_clock();
      const size_t i = base + lane;
      if (i < n) {
        uint32_t s[16], m[8], o[16];
        load_words(sigs, i, 16, s);
        load_words(msgs, i, 8, m);
        const uint8_t st = ecdsa_recover<K1Traits, true>(s, m, gtab, o);
        store_words(out, i, 16, o);
        status[i] = st;
      }
      __syncwarp();
      if (lane == 0) {
        times[2 * (base / 32)] = t0;
        times[2 * (base / 32) + 1] = phase_clock();
      }
    }
  }
}

// one 256-thread block per SM (counter: one zeroed word)
cudaError_t launch_k1_phase(bool sync, const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* gtab, uint8_t* out,
                            uint8_t* status, unsigned long long* counter, unsigned long long* times, int num_sms, cudaStream_t stream) {
  if (sync) k1_phase_kernel<true><<<num_sms, 256, 0, stream>>>(sigs, msgs, n, gtab, out, status, counter, times);
  else k1_phase_kernel<false><<<num_sms, 256, 0, stream>>>(sigs, msgs, n, gtab, out, status, counter, times);
  return cudaGetLastError();
}

// A secp256k1 batch too small to fill the GPU, in one-warp blocks spread over
// the SMs: a lane pair per signature while that takes at most two warps per SM
// (a signature then finishes in 0.84 of the time), one lane above
cudaError_t launch_plain_k1_small(const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* gtab, uint8_t* out, uint8_t* status,
                                  int num_sms, cudaStream_t stream) {
  const int lanes = 2 * n <= (size_t)num_sms * 64 ? 2 : 1;
  return launch_k1_lanes(lanes, sigs, msgs, n, 32, gtab, out, status, stream);
}

}  // namespace sg
