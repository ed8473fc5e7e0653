// Allocation-free variant of the batched mixed-curve call.
//
// Some callers cannot allocate device memory per call: processes whose GPU
// memory is owned by another allocator (a framework's caching allocator, or a
// pool reserved at start-up with a fixed budget), and latency-critical verifier
// threads that cannot afford cudaMalloc's implicit device synchronisation or
// its failure modes under memory pressure.  sigops_verify_mixed_noalloc serves
// them: it needs no context and calls no cudaMalloc / cudaFree.  Its scratch
// (per-curve counters and index lists), the generator tables and the device
// error word live in the file-scope static __device__ arrays below, which every
// GPU that loads the library holds until the process exits: about 0.75 MiB of
// scratch and 9 MiB of generator tables (16-bit windows: 4 MiB for secp256k1
// with its 2^128 G half, 2 MiB for P-256, 3 MiB for ed25519).  These arrays
// are separate from the tables each context allocates; under
// CUDA_MODULE_LOADING=EAGER every GPU of the process holds them even when this
// entry point is never called (under the default lazy loading, from the first
// use of the module's kernels).
//
// The first call on each device performs a one-time set-up with that device
// current: cudaGetSymbolAddress for each array (host code must not use the
// arrays' names as device addresses: on the host they are only stand-ins) and
// an upload of the tables with cudaMemcpyToSymbol, followed by a device
// synchronisation so that no kernel on a non-blocking stream can read a table
// before it has landed.  Make that first call before any stream capture.  All
// calls share the arrays and each call clears the counters it needs, so calls
// whose work overlaps on the GPU (different streams, or different host
// threads) race with each other: serialise them.  A device-side error of these
// calls sets the static error word; sigops_noalloc_status reads and clears it.
#include <cuda_runtime.h>

#include <deque>
#include <mutex>

#include "../../include/sigops.h"
#include "batched.cuh"

namespace {

constexpr size_t kMaxItems = SIGOPS_NOALLOC_MAX_ITEMS;
// the fused kernel with one 32-item tile per warp (one launch, no side streams)
constexpr int kVariant = 1;
constexpr size_t kScratchHead = 256;  // Scratch record, padded to the array's alignment
constexpr size_t kScratchBytes = kScratchHead + 3 * kMaxItems * sizeof(uint32_t);

static_assert(sizeof(sg::Scratch) <= kScratchHead, "scratch record fits its slot");

static __device__ __align__(256) uint8_t g_noalloc_scratch[kScratchBytes];
static __device__ __align__(256) uint32_t g_noalloc_tab_k1[2 * sg::ECDSA_GTAB * 16];
static __device__ __align__(256) uint32_t g_noalloc_tab_r1[sg::ECDSA_GTAB * 16];
static __device__ __align__(256) uint32_t g_noalloc_tab_ed[sg::ED_GTAB * 24];
static __device__ uint32_t g_noalloc_err;

struct DeviceSetup {
  bool ready = false;
  uint8_t* scratch = nullptr;  // device address of g_noalloc_scratch
  uint32_t* tab[3] = {nullptr, nullptr, nullptr};
  uint32_t* err = nullptr;
  int grid = 0;
  int num_sms = 0;
};

// one record per device; a deque never moves its elements when it grows, and
// callers get a copy taken under the lock
std::mutex g_mu;
std::deque<DeviceSetup> g_dev;

// once per device, with the device current; allocates no device memory
int setup(int device, DeviceSetup* out) {
  std::lock_guard<std::mutex> g(g_mu);
  while ((int)g_dev.size() <= device) g_dev.emplace_back();
  DeviceSetup& d = g_dev[device];
  if (d.ready) {
    *out = d;
    return SIGOPS_OK;
  }
  if (cudaGetSymbolAddress((void**)&d.scratch, g_noalloc_scratch) != cudaSuccess) return SIGOPS_E_CUDA;
  if (cudaGetSymbolAddress((void**)&d.tab[0], g_noalloc_tab_k1) != cudaSuccess) return SIGOPS_E_CUDA;
  if (cudaGetSymbolAddress((void**)&d.tab[1], g_noalloc_tab_r1) != cudaSuccess) return SIGOPS_E_CUDA;
  if (cudaGetSymbolAddress((void**)&d.tab[2], g_noalloc_tab_ed) != cudaSuccess) return SIGOPS_E_CUDA;
  if (cudaGetSymbolAddress((void**)&d.err, g_noalloc_err) != cudaSuccess) return SIGOPS_E_CUDA;
  // generator tables, built on the host with the kernels' own arithmetic
  const sg::KernelTables& h = sg::kernel_tables();
  static_assert(sizeof g_noalloc_tab_k1 == 2 * sg::ECDSA_GTAB * 16 * 4 && sizeof g_noalloc_tab_ed == sg::ED_GTAB * 24 * 4, "table sizes");
  uint32_t zero = 0;
  if (cudaMemcpyToSymbol(g_noalloc_tab_k1, h.tab[0].data(), sizeof g_noalloc_tab_k1) != cudaSuccess ||
      cudaMemcpyToSymbol(g_noalloc_tab_r1, h.tab[1].data(), sizeof g_noalloc_tab_r1) != cudaSuccess ||
      cudaMemcpyToSymbol(g_noalloc_tab_ed, h.tab[2].data(), sizeof g_noalloc_tab_ed) != cudaSuccess ||
      cudaMemcpyToSymbol(g_noalloc_err, &zero, sizeof zero) != cudaSuccess)
    return SIGOPS_E_CUDA;
  // a pageable upload may return before its data has landed, and the first
  // launch may go to a non-blocking stream that does not wait for it
  if (cudaDeviceSynchronize() != cudaSuccess) return SIGOPS_E_CUDA;
  if (cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return SIGOPS_E_CUDA;
  int bps = sg::batched_max_blocks_per_sm(kVariant);
  if (bps <= 0) return SIGOPS_E_CUDA;
  d.grid = d.num_sms * bps;
  d.ready = true;
  *out = d;
  return SIGOPS_OK;
}

}  // namespace

extern "C" int sigops_verify_mixed_noalloc(const uint8_t* d_curves, const uint8_t* d_sigs, const uint8_t* d_msgs, const uint8_t* d_pks,
                                           size_t n, uint8_t* d_out, uint8_t* d_status, void* stream) {
  if (n == 0) return SIGOPS_OK;
  if (n > kMaxItems) return SIGOPS_E_RANGE;
  if (!d_curves || !d_sigs || !d_msgs || !d_pks || !d_out || !d_status) return SIGOPS_E_INVAL;
  auto misaligned = [](const void* p) { return ((uintptr_t)p & 15u) != 0; };
  if (misaligned(d_sigs) || misaligned(d_msgs) || misaligned(d_pks) || misaligned(d_out)) return SIGOPS_E_INVAL;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return SIGOPS_E_NODEV;
  DeviceSetup d;
  int rc = setup(device, &d);
  if (rc != SIGOPS_OK) return rc;
  const size_t cg = (n + 255) / 256;
  const int classify_grid = (int)(cg < (size_t)d.num_sms * 8 ? cg : (size_t)d.num_sms * 8);
  // the per-curve index lists follow the counters; launch_batched clears the counters
  uint32_t* idx = reinterpret_cast<uint32_t*>(d.scratch + kScratchHead);
  const sg::GenTables tabs{{d.tab[0], d.tab[1], d.tab[2]}, {nullptr, nullptr, nullptr}};  // the fused variant reads the 16-bit tables only
  cudaError_t e = sg::launch_batched(d_curves, d_sigs, d_msgs, d_pks, n, d_out, d_status, idx, d.scratch, nullptr, tabs, d.err, d.grid, kVariant,
                                     classify_grid, nullptr, (cudaStream_t)stream);
  return e == cudaSuccess ? SIGOPS_OK : SIGOPS_E_CUDA;
}

extern "C" int sigops_noalloc_status(void* stream) {
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return SIGOPS_E_NODEV;
  DeviceSetup d;
  {
    std::lock_guard<std::mutex> g(g_mu);
    if (device >= (int)g_dev.size() || !g_dev[device].ready) return SIGOPS_OK;  // no call has run on this device
    d = g_dev[device];
  }
  // read after the work queued on `stream`, then clear when set
  uint32_t e = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(&e, d.err, sizeof e, cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
    return SIGOPS_E_CUDA;
  if (e == 0) return SIGOPS_OK;
  if (cudaMemsetAsync(d.err, 0, sizeof e, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) return SIGOPS_E_CUDA;
  return SIGOPS_E_TIMEDOUT;
}
