// Internal launch interface between the kernels and the host runtime.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

struct sigops_ctx;

namespace sg {

constexpr int PLAIN_BLOCK = 256;  // workload-generation kernels

// error bits reported through the device error word
enum : uint32_t { DEV_ERR_WAIT_TIMEOUT = 1u, DEV_ERR_MISALIGNED = 2u, DEV_ERR_QUEUE_TIMEOUT = 4u };

// plain kernels: one item per thread, the grid sized to the batch.  Variants:
// 0 = 256-thread blocks, one per SM (no register cap); 1 = two per SM (128
// registers); 2 = 128-thread blocks, three per SM (170 registers).
constexpr int PLAIN_VARIANTS = 3;
inline int plain_variant_block(int variant) { return variant == 2 ? 128 : 256; }
cudaError_t launch_plain(int curve, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, const uint32_t* gtab,
                         uint8_t* out, uint8_t* status, uint32_t* err, int variant, cudaStream_t stream);
int plain_max_blocks_per_sm(int curve, int variant);
// a batch of at most 320 signatures per SM (10 warps: one partial wave of the
// tuned kernels, which would pile whole blocks onto some SMs): one-warp blocks
// spread evenly over the SMs, secp256k1 with a lane pair per signature while
// that takes at most two warps per SM (k_split.cu, k_r1.cu, k_ed.cu)
inline bool plain_small_batch(size_t n, int num_sms) { return n <= (size_t)num_sms * 320; }
cudaError_t launch_plain_small(int curve, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, const uint32_t* gtab,
                               uint8_t* out, uint8_t* status, uint32_t* err, int num_sms, cudaStream_t stream);
cudaError_t launch_plain_k1_small(const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* gtab, uint8_t* out, uint8_t* status,
                                  int num_sms, cudaStream_t stream);
cudaError_t launch_plain_r1_small(const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* gtab, uint8_t* out, uint8_t* status,
                                  uint32_t* err, cudaStream_t stream);
cudaError_t launch_plain_ed_small(const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, const uint32_t* btab,
                                  uint8_t* valid, uint8_t* status, uint32_t* err, cudaStream_t stream);
cudaError_t launch_plain_k1(const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* gtab, uint8_t* out, uint8_t* status,
                            uint32_t* err, int variant, cudaStream_t stream);
cudaError_t launch_plain_r1(const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* gtab, uint8_t* out, uint8_t* status,
                            uint32_t* err, int variant, cudaStream_t stream);
cudaError_t launch_plain_ed(const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, const uint32_t* btab, uint8_t* valid,
                            uint8_t* status, uint32_t* err, int variant, cudaStream_t stream);
cudaError_t launch_raw_ed(const uint8_t* sigs, const uint8_t* msgs, const uint64_t* offsets, const uint32_t* lens, const uint8_t* pks,
                          size_t n, const uint32_t* btab, uint8_t* valid, uint8_t* status, uint32_t* err, int variant,
                          cudaStream_t stream);
int occupancy_plain_k1(int variant);
int occupancy_plain_r1(int variant);
int occupancy_plain_ed(int variant);
cudaError_t launch_sign_ecdsa(int curve, const uint8_t* secrets, const uint8_t* nonces, const uint8_t* msgs, size_t n, const uint32_t* gtab,
                              uint8_t* sigs, uint8_t* pubs, uint8_t* status, uint32_t* err, int grid, cudaStream_t stream);
cudaError_t launch_sign_ed(const uint8_t* seeds, const uint8_t* msgs, size_t n, const uint32_t* btab, uint8_t* sigs, uint8_t* pks,
                           uint32_t* err, int grid, cudaStream_t stream);
// batched mixed-curve engine: scratch = Scratch record + 3*n u32 index lists.
// variants 0..3: the fused kernel (0 = persistent, 256 threads x 1 block/SM;
// 1 = one tile per warp, 256 threads; 2 = one tile per warp, 128 x 3;
// 3 = one tile per warp, 256 x 2); variants 4 + a + 8 b + 64 c (4..515): three
// single-curve pipelines (secp256k1 in configuration a, P-256 in b, ed25519
// in c).  Configurations (block x blocks per SM / register budget, per-point
// window WR, generator window WG):
//   0: 256 x 1 / 255, 1: 128 x 3 / 170, 2: 256 x 2 / 128, 3: 64 / 144,
//   4: 512 x 1 / 128 (all WR 5, WG 16, tables in global memory);
//   5: as 1 with WR 4 (half the per-signature table: 12 warps' stacks stay in
//   L2); 6: as 2 with WR 6; 7: as 2 with WG 8 (tables staged into shared
//   memory by a bulk copy).
constexpr int BATCHED_FUSED_VARIANTS = 4;
constexpr int CURVE_CONFIGS = 8;
constexpr int BATCHED_VARIANTS = BATCHED_FUSED_VARIANTS + CURVE_CONFIGS * CURVE_CONFIGS * CURVE_CONFIGS;
inline int split_variant(int a, int b, int c) { return BATCHED_FUSED_VARIANTS + a + CURVE_CONFIGS * b + CURVE_CONFIGS * CURVE_CONFIGS * c; }
// configuration of curve c (0..2) in a single-curve variant
inline int split_config(int variant, int c) {
  int v = variant - BATCHED_FUSED_VARIANTS;
  for (int k = 0; k < c; ++k) v /= CURVE_CONFIGS;
  return v % CURVE_CONFIGS;
}
// block size, window widths of a configuration
int curve_config_block(int config);
void curve_config_windows(int config, int* wr, int* wg);
// blocks per SM of curve c's kernel in a configuration
int curve_config_occupancy(int c, int config);
// device pointers of the generator tables: 16-bit windows (global memory) and
// 8-bit windows (staged into shared memory), per curve
struct GenTables {
  const uint32_t* big[3];
  const uint32_t* small[3];
};
int batched_variant_block(int variant);
int batched_max_blocks_per_sm(int variant);
size_t batched_scratch_bytes();
// the single-curve variants' shared-inversion scratch for n items (16-byte
// aligned, item-indexed: r^-1 then the result points)
size_t batched_defer_bytes(size_t n);
// side streams and events on which the single-curve kernels run beside each
// other (fork after the classify kernel, join before returning); without them
// the three kernels run one after another on the caller's stream
struct ForkStreams {
  cudaStream_t aux[2];
  cudaEvent_t ev[3];
};
// priority: as cudaStreamCreateWithPriority (0 = default)
cudaError_t fork_streams_create(ForkStreams* f, int priority = 0);
void fork_streams_destroy(ForkStreams* f);
// grid: blocks of the fused kernel (the single-curve kernels size their grids
// to the batch: one item per thread).  defer: batched_defer_bytes(n) of
// scratch, required by the single-curve variants (NULL for the fused ones)
cudaError_t launch_batched(const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, uint8_t* out,
                           uint8_t* status, uint32_t* idx, void* scratch, void* defer, const GenTables& tabs, uint32_t* err, int grid,
                           int variant, int classify_grid, const ForkStreams* fork, cudaStream_t stream);
// secp256k1 recovery by 1 or 2 lanes per signature (k_split.cu)
cudaError_t launch_k1_lanes(int lanes, const uint8_t* sigs, const uint8_t* msgs, size_t n, int block, const uint32_t* gtab,
                            uint8_t* out, uint8_t* status, cudaStream_t stream);
// secp256k1 recovery by persistent warps, free-running or block-synchronised,
// with per-group timings (k_split.cu)
cudaError_t launch_k1_phase(bool sync, const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* gtab, uint8_t* out,
                            uint8_t* status, unsigned long long* counter, unsigned long long* times, int num_sms, cudaStream_t stream);

// Record the calling thread's last-error message (sigops_last_error) and
// return code (host.cu).
int report(int code, const char* what);

// Device and pinned host allocations of the library (host.cu).  A test hook
// (sigops_test_fail_allocations) makes the next ones fail as if out of memory.
cudaError_t dev_alloc(void** p, size_t bytes);
void dev_free(void* p);
cudaError_t host_alloc(void** p, size_t bytes, unsigned flags = cudaHostAllocDefault);
void host_free(void* p);

// what the serving loop needs from a context (host.cu)
struct CtxView {
  int device;
  int num_sms;
  const uint32_t* gtab[3];
  GenTables tabs;
  uint32_t* d_err;
  int batched_grid;
  int batched_variant;
};
int ctx_view(sigops_ctx* c, CtxView* v);
// cached autotuner choice for this device (autotune.cu): variants of the three
// plain kernels and the batched kernel; false when there is none
bool tune_cache_lookup(int device, int variants[4]);

cudaError_t launch_field_test(int field, int op, const void* a, const void* b, void* out, int n, cudaStream_t stream);
cudaError_t launch_sha512_test(const void* in, void* out, int n, cudaStream_t stream);
cudaError_t launch_imad_probe(uint32_t* out, uint32_t iters, int grid, int block, cudaStream_t stream);
cudaError_t launch_wait_expiry(uint32_t max_polls, uint32_t* err, cudaStream_t stream);
cudaError_t launch_mul_probe(int form, uint32_t* out, uint32_t iters, int grid, int block, cudaStream_t stream);

}  // namespace sg
