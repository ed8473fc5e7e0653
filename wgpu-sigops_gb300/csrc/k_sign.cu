// Workload-generation kernels: batch signing on the device.
#include "kernels.cuh"
#include "sign.cuh"

namespace sg {

template <class T>
__global__ void __launch_bounds__(PLAIN_BLOCK) ecdsa_sign_kernel(const uint8_t* __restrict__ secrets, const uint8_t* __restrict__ nonces,
                                                                  const uint8_t* __restrict__ msgs, size_t n, const uint32_t* __restrict__ gtab,
                                                                  uint8_t* __restrict__ sigs, uint8_t* __restrict__ pubs, uint8_t* __restrict__ status,
                                                                  uint32_t* err) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint32_t d[8], k[8], m[8], s[16], p[16];
    load_words(secrets, i, 8, d);
    load_words(nonces, i, 8, k);
    load_words(msgs, i, 8, m);
    uint8_t st = ecdsa_sign<T>(d, k, m, gtab, s, p);
    store_words(sigs, i, 16, s);
    store_words(pubs, i, 16, p);
    status[i] = st;
  }
}

__global__ void __launch_bounds__(PLAIN_BLOCK) ed_sign_kernel(const uint8_t* __restrict__ seeds, const uint8_t* __restrict__ msgs, size_t n,
                                                               const uint32_t* __restrict__ btab, uint8_t* __restrict__ sigs,
                                                               uint8_t* __restrict__ pks, uint32_t* err) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint32_t sd[8], m[8], s[16], p[8];
    load_words(seeds, i, 8, sd);
    load_words(msgs, i, 8, m);
    ed25519_sign(sd, m, btab, s, p);
    store_words(sigs, i, 16, s);
    store_words(pks, i, 8, p);
  }
}

cudaError_t launch_sign_ecdsa(int curve, const uint8_t* secrets, const uint8_t* nonces, const uint8_t* msgs, size_t n, const uint32_t* gtab,
                              uint8_t* sigs, uint8_t* pubs, uint8_t* status, uint32_t* err, int grid, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  if (curve == CURVE_SECP256K1)
    ecdsa_sign_kernel<K1Traits><<<grid, PLAIN_BLOCK, 0, stream>>>(secrets, nonces, msgs, n, gtab, sigs, pubs, status, err);
  else if (curve == CURVE_SECP256R1)
    ecdsa_sign_kernel<R1Traits><<<grid, PLAIN_BLOCK, 0, stream>>>(secrets, nonces, msgs, n, gtab, sigs, pubs, status, err);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_sign_ed(const uint8_t* seeds, const uint8_t* msgs, size_t n, const uint32_t* btab, uint8_t* sigs, uint8_t* pks,
                           uint32_t* err, int grid, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  ed_sign_kernel<<<grid, PLAIN_BLOCK, 0, stream>>>(seeds, msgs, n, btab, sigs, pks, err);
  return cudaGetLastError();
}

}  // namespace sg
