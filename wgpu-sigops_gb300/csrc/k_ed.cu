// Plain ed25519 verification kernel instantiation.
#include "plain.cuh"

namespace sg {

// one item per thread
template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) ed_plain_kernel(const uint8_t* __restrict__ sigs, const uint8_t* __restrict__ msgs,
                                                          const uint8_t* __restrict__ pks, size_t n, const uint32_t* __restrict__ btab,
                                                          uint8_t* __restrict__ valid, uint8_t* __restrict__ status, uint32_t* err) {
  const size_t i = (size_t)blockIdx.x * BLOCK + threadIdx.x;
  if (i >= n) return;
  uint32_t s[16], m[8], p[8];
  load_words(sigs, i, 16, s);
  load_words(msgs, i, 8, m);
  load_words(pks, i, 8, p);
  uint8_t st = ed25519_verify(s, m, p, btab);
  valid[i] = st == ST_OK;
  status[i] = st;
}

// ed25519 over messages of any length: message i is msgs[offsets[i] ..
// offsets[i] + lens[i]) (no alignment needed)
template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) ed_raw_kernel(const uint8_t* __restrict__ sigs, const uint8_t* __restrict__ msgs,
                                                        const uint64_t* __restrict__ offsets, const uint32_t* __restrict__ lens,
                                                        const uint8_t* __restrict__ pks, size_t n, const uint32_t* __restrict__ btab,
                                                        uint8_t* __restrict__ valid, uint8_t* __restrict__ status, uint32_t* err) {
  const size_t i = (size_t)blockIdx.x * BLOCK + threadIdx.x;
  if (i >= n) return;
  uint32_t s[16], p[8];
  load_words(sigs, i, 16, s);
  load_words(pks, i, 8, p);
  uint8_t st = ed25519_verify_raw(s, msgs + offsets[i], lens[i], p, btab);
  valid[i] = st == ST_OK;
  status[i] = st;
}

cudaError_t launch_raw_ed(const uint8_t* sigs, const uint8_t* msgs, const uint64_t* offsets, const uint32_t* lens, const uint8_t* pks,
                          size_t n, const uint32_t* btab, uint8_t* valid, uint8_t* status, uint32_t* err, int variant,
                          cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  const int block = plain_variant_block(variant);
  const unsigned grid = (unsigned)((n + block - 1) / block);
  if (variant == 1) ed_raw_kernel<256, 2><<<grid, 256, 0, stream>>>(sigs, msgs, offsets, lens, pks, n, btab, valid, status, err);
  else if (variant == 2) ed_raw_kernel<128, 3><<<grid, 128, 0, stream>>>(sigs, msgs, offsets, lens, pks, n, btab, valid, status, err);
  else ed_raw_kernel<256, 1><<<grid, 256, 0, stream>>>(sigs, msgs, offsets, lens, pks, n, btab, valid, status, err);
  return cudaGetLastError();
}

cudaError_t launch_plain_ed(const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, const uint32_t* btab, uint8_t* valid,
                            uint8_t* status, uint32_t* err, int variant, cudaStream_t stream) {
  const int block = plain_variant_block(variant);
  const unsigned grid = (unsigned)((n + block - 1) / block);
  if (variant == 1) ed_plain_kernel<256, 2><<<grid, 256, 0, stream>>>(sigs, msgs, pks, n, btab, valid, status, err);
  else if (variant == 2) ed_plain_kernel<128, 3><<<grid, 128, 0, stream>>>(sigs, msgs, pks, n, btab, valid, status, err);
  else ed_plain_kernel<256, 1><<<grid, 256, 0, stream>>>(sigs, msgs, pks, n, btab, valid, status, err);
  return cudaGetLastError();
}

// a batch too small to fill the GPU: one warp per block, spread over the SMs
cudaError_t launch_plain_ed_small(const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, const uint32_t* btab,
                                  uint8_t* valid, uint8_t* status, uint32_t* err, cudaStream_t stream) {
  ed_plain_kernel<32, 1><<<(unsigned)((n + 31) / 32), 32, 0, stream>>>(sigs, msgs, pks, n, btab, valid, status, err);
  return cudaGetLastError();
}

int occupancy_plain_ed(int variant) {
  int b = 0;
  if (variant == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ed_plain_kernel<256, 2>, 256, 0);
  else if (variant == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ed_plain_kernel<128, 3>, 128, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ed_plain_kernel<256, 1>, 256, 0);
  return b;
}

}  // namespace sg
