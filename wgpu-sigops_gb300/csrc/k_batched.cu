// Batched mixed-curve engine: kernel instantiations and launchers.
#include "batched.cuh"

namespace sg {

template <int BLOCK>
static int occ() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_kernel<BLOCK>, BLOCK, 0);
  return b;
}

int batched_max_blocks_per_sm(int block) {
  switch (block) {
    case 128: return occ<128>();
    case 256: return occ<256>();
    default: return 0;
  }
}

cudaError_t launch_batched(const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, uint8_t* out,
                           uint8_t* status, uint32_t* idx, void* scratch, const uint32_t* gk1, const uint32_t* gr1, const uint32_t* ged,
                           uint32_t* err, int grid, int block, int classify_grid, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  Scratch* sc = (Scratch*)scratch;
  cudaError_t e = cudaMemsetAsync(sc, 0, sizeof(Scratch), stream);
  if (e != cudaSuccess) return e;
  classify_kernel<<<classify_grid, 256, 0, stream>>>(curves, n, idx, sc);
  MixedIO io{curves, sigs, msgs, pks, out, status, n};
  BatchTables t{gk1, gr1, ged};
  switch (block) {
    case 128: batched_kernel<128><<<grid, 128, 0, stream>>>(io, idx, t, sc, err); break;
    case 256: batched_kernel<256><<<grid, 256, 0, stream>>>(io, idx, t, sc, err); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

size_t batched_scratch_bytes() { return sizeof(Scratch); }

}  // namespace sg
