// Autotuner: picks the fastest launch variant of each kernel on this device.
//
// No counterpart in the reference (its launch shape is fixed at 256-thread
// workgroups, src/benchmarks/mod.rs:10-53).  A probe batch with the 40/30/30
// curve mix is signed on the device (valid signatures, so every item runs the
// full path).  Each curve's plain kernel is timed per variant with CUDA events
// (one warm-up, best of three).  The batched engine is tuned in two stages: all
// variants once on an 8-wave prefix of the probe (the prefix keeps the curve
// mix: items are interleaved 4:3:3), then the twelve fastest again on the whole
// probe, best of three.  The ranking of the concurrent single-curve kernels
// depends on the batch size, so the probe should be as large as the batches
// the caller runs.  The search space is the compiled variants: for each curve,
// block shape and register budget (256 x 1, 128 x 3, 256 x 2, 64, 512 x 1),
// per-point window width (4, 5, 6 bits) and generator window width (16 bits
// with tables in global memory, 8 bits with tables staged into shared memory
// by a bulk copy); the fused mixed-curve kernel in four shapes.
//
// Results can be kept in a cache file (SIGOPS_TUNE_CACHE, one line per device
// name and SM count) that sigops_create reads back.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sigops.h"
#include "launch.h"

namespace {

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

void fill_random(std::vector<uint8_t>& v, uint64_t& s) {
  for (size_t i = 0; i < v.size(); i += 8) {
    uint64_t r = splitmix(s);
    for (size_t k = 0; k < 8 && i + k < v.size(); ++k) v[i + k] = (uint8_t)(r >> (8 * k));
  }
}

// dst row i = src row perm[i]
__global__ void gather_rows_kernel(uint8_t* __restrict__ dst, const uint8_t* __restrict__ src, const uint32_t* __restrict__ perm, size_t n,
                                   uint32_t row) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint8_t* s = src + (size_t)perm[i] * row;
    uint8_t* d = dst + i * row;
    for (uint32_t k = 0; k < row; ++k) d[k] = s[k];
  }
}

struct DevBuf {
  uint8_t* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

std::string cache_key(int device) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return "";
  char buf[300];
  snprintf(buf, sizeof buf, "%s|sm%d|%s", prop.name, prop.multiProcessorCount, sigops_version());
  return buf;
}

std::mutex g_cache_mu;

}  // namespace

namespace sg {

// read a cached tuning for this device: fills variants[4]; false if none
bool tune_cache_lookup(int device, int variants[4]) {
  const char* path = getenv("SIGOPS_TUNE_CACHE");
  if (!path || !*path) return false;
  std::lock_guard<std::mutex> g(g_cache_mu);
  FILE* f = fopen(path, "r");
  if (!f) return false;
  std::string key = cache_key(device);
  char line[512];
  bool found = false;
  while (fgets(line, sizeof line, f)) {
    char* tab = strchr(line, '\t');
    if (!tab) continue;
    *tab = 0;
    if (key == line && sscanf(tab + 1, "%d %d %d %d", &variants[0], &variants[1], &variants[2], &variants[3]) == 4) found = true;
  }
  fclose(f);
  return found;
}

static void tune_cache_store(int device, const int variants[4]) {
  const char* path = getenv("SIGOPS_TUNE_CACHE");
  if (!path || !*path) return;
  std::lock_guard<std::mutex> g(g_cache_mu);
  std::string key = cache_key(device);
  std::vector<std::string> keep;
  if (FILE* f = fopen(path, "r")) {
    char line[512];
    while (fgets(line, sizeof line, f)) {
      std::string s(line);
      if (s.compare(0, key.size() + 1, key + "\t") != 0) keep.push_back(s);
    }
    fclose(f);
  }
  if (FILE* f = fopen(path, "w")) {
    for (auto& s : keep) fputs(s.c_str(), f);
    fprintf(f, "%s\t%d %d %d %d\n", key.c_str(), variants[0], variants[1], variants[2], variants[3]);
    fclose(f);
  }
}

}  // namespace sg

extern "C" int sigops_autotune(sigops_ctx* ctx, size_t probe_items, char* report, size_t report_cap) {
  sg::CtxView v;
  if (!ctx || sg::ctx_view(ctx, &v) != SIGOPS_OK) return SIGOPS_E_INVAL;
  if (probe_items == 0) probe_items = (size_t)v.num_sms * 256 * 16;
  const size_t n = probe_items;
  cudaSetDevice(v.device);
  // probe batch: 40/30/30 by position
  const size_t n1 = n * 4 / 10, n2 = n * 3 / 10, n3 = n - n1 - n2;
  std::vector<uint8_t> curves(n), secrets(n * 32), nonces(n * 32), msgs(n * 32), seeds(n * 32);
  uint64_t s = 0x5349474f5053ull;
  fill_random(secrets, s);
  fill_random(nonces, s);
  fill_random(msgs, s);
  fill_random(seeds, s);
  for (size_t i = 0; i < n; ++i) curves[i] = i < n1 ? 0 : (i < n1 + n2 ? 1 : 2);
  // interleaved order for the batched engine: every prefix keeps the 4:3:3 mix
  std::vector<uint32_t> perm;
  perm.reserve(n);
  {
    static const int pat[10] = {0, 1, 2, 0, 1, 2, 0, 0, 1, 2};
    size_t next[3] = {0, n1, n1 + n2};
    const size_t end[3] = {n1, n1 + n2, n};
    for (size_t i = 0; perm.size() < n; ++i) {
      int c = pat[i % 10];
      for (int t = 0; t < 3 && next[c] == end[c]; ++t) c = (c + 1) % 3;
      perm.push_back((uint32_t)next[c]++);
    }
  }
  DevBuf d;
  const size_t pad = 256 * ((n + 255) / 256);
  const size_t o_cur = 0, o_sec = pad, o_non = o_sec + n * 32, o_msg = o_non + n * 32, o_seed = o_msg + n * 32,
               o_sig = o_seed + n * 32, o_pub = o_sig + n * 64, o_pk = o_pub + n * 64, o_out = o_pk + n * 32, o_st = o_out + n * 64,
               o_idx = o_st + pad, o_scr = o_idx + 3 * n * 4, o_perm = o_scr + 256, o_icur = o_perm + 4 * pad, o_isig = o_icur + pad,
               o_imsg = o_isig + n * 64, o_ipk = o_imsg + n * 32, o_def = o_ipk + n * 32, total = o_def + sg::batched_defer_bytes(n);
  if (cudaMalloc(&d.p, total) != cudaSuccess) return SIGOPS_E_NOMEM;
  cudaStream_t st;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return SIGOPS_E_CUDA;
  cudaMemcpyAsync(d.p + o_cur, curves.data(), n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d.p + o_sec, secrets.data(), n * 32, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d.p + o_non, nonces.data(), n * 32, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d.p + o_msg, msgs.data(), n * 32, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d.p + o_seed, seeds.data(), n * 32, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(d.p + o_pk, 0, n * 32, st);
  const int sign_grid = v.num_sms * 2;
  sg::launch_sign_ecdsa(0, d.p + o_sec, d.p + o_non, d.p + o_msg, n1, v.gtab[0], d.p + o_sig, d.p + o_pub, d.p + o_st, v.d_err, sign_grid, st);
  sg::launch_sign_ecdsa(1, d.p + o_sec + n1 * 32, d.p + o_non + n1 * 32, d.p + o_msg + n1 * 32, n2, v.gtab[1], d.p + o_sig + n1 * 64,
                        d.p + o_pub + n1 * 64, d.p + o_st + n1, v.d_err, sign_grid, st);
  sg::launch_sign_ed(d.p + o_seed + (n1 + n2) * 32, d.p + o_msg + (n1 + n2) * 32, n3, v.gtab[2], d.p + o_sig + (n1 + n2) * 64,
                     d.p + o_pk + (n1 + n2) * 32, v.d_err, sign_grid, st);
  cudaMemcpyAsync(d.p + o_perm, perm.data(), n * 4, cudaMemcpyHostToDevice, st);
  {
    const uint32_t* pm = (const uint32_t*)(d.p + o_perm);
    const int gg = v.num_sms * 4;
    gather_rows_kernel<<<gg, 256, 0, st>>>(d.p + o_icur, d.p + o_cur, pm, n, 1);
    gather_rows_kernel<<<gg, 256, 0, st>>>(d.p + o_isig, d.p + o_sig, pm, n, 64);
    gather_rows_kernel<<<gg, 256, 0, st>>>(d.p + o_imsg, d.p + o_msg, pm, n, 32);
    gather_rows_kernel<<<gg, 256, 0, st>>>(d.p + o_ipk, d.p + o_pk, pm, n, 32);
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    cudaStreamDestroy(st);
    return SIGOPS_E_CUDA;
  }
  sg::ForkStreams fork;
  if (sg::fork_streams_create(&fork) != cudaSuccess) {
    sg::fork_streams_destroy(&fork);
    cudaStreamDestroy(st);
    return SIGOPS_E_CUDA;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto off_of = [&](int c) { return c == 0 ? (size_t)0 : c == 1 ? n1 : n1 + n2; };
  auto cnt_of = [&](int c) { return c == 0 ? n1 : c == 1 ? n2 : n3; };
  auto time_it = [&](auto&& launch, int reps = 3) -> float {
    launch();
    float best = 1e30f;
    for (int r = 0; r < reps; ++r) {
      cudaEventRecord(e0, st);
      launch();
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      best = std::min(best, ms);
    }
    return cudaGetLastError() == cudaSuccess ? best : 1e30f;
  };
  std::string rep = "{";
  int chosen[4] = {0, 0, 0, 0};
  // batched engine.  Stage 0: each curve's single-curve pipeline alone, in
  // each of its configurations (launch shape, register budget, window widths),
  // on that curve's items of the probe.  Stage 1: the fused variants and every
  // combination of the three best configurations per curve once on a prefix of
  // the interleaved probe.  Stage 2: the twelve fastest on the whole probe,
  // best of three.
  {
    const size_t n_short = std::min(n, (size_t)v.num_sms * 256 * 8);
    auto run_batched = [&](int var, size_t first, size_t items, bool interleaved, int reps) {
      const int grid = v.num_sms * sg::batched_max_blocks_per_sm(var);
      const int classify_grid = (int)std::min((items + 255) / 256, (size_t)v.num_sms * 8);
      const size_t ic = interleaved ? o_icur : o_cur, is = interleaved ? o_isig : o_sig, im = interleaved ? o_imsg : o_msg,
                   ip = interleaved ? o_ipk : o_pk;
      return time_it(
          [&] {
            sg::launch_batched(d.p + ic + first, d.p + is + first * 64, d.p + im + first * 32, d.p + ip + first * 32, items, d.p + o_out,
                               d.p + o_st, (uint32_t*)(d.p + o_idx), d.p + o_scr, d.p + o_def, v.tabs, v.d_err, grid, var, classify_grid,
                               &fork, st);
          },
          reps);
    };
    static const char* kCurve[3] = {"secp256k1", "secp256r1", "ed25519"};
    rep += "\"curve_configs\": {";
    std::vector<int> best_cfg[3];
    for (int c = 0; c < 3; ++c) {
      std::vector<std::pair<float, int>> times;
      char b[160];
      snprintf(b, sizeof b, "%s\"%s\": {", c ? ", " : "", kCurve[c]);
      rep += b;
      bool firstc = true;
      for (int cfg = 0; cfg < sg::CURVE_CONFIGS; ++cfg) {
        const int var = sg::split_variant(cfg, cfg, cfg);  // the other curves have no items here
        if (sg::curve_config_occupancy(c, cfg) <= 0 || cnt_of(c) == 0) continue;
        const float ms = run_batched(var, off_of(c), cnt_of(c), false, 2);
        times.push_back({ms, cfg});
        int wr, wg;
        sg::curve_config_windows(cfg, &wr, &wg);
        snprintf(b, sizeof b, "%s\"%d\": {\"ms\": %.3f, \"block\": %d, \"blocks_per_sm\": %d, \"wr\": %d, \"wg\": %d}",
                 firstc ? "" : ", ", cfg, ms, sg::curve_config_block(cfg), sg::curve_config_occupancy(c, cfg), wr, wg);
        firstc = false;
        rep += b;
      }
      rep += "}";
      std::sort(times.begin(), times.end());
      for (size_t k = 0; k < times.size() && k < 3; ++k) best_cfg[c].push_back(times[k].second);
      if (best_cfg[c].empty()) best_cfg[c].push_back(2);
    }
    rep += "}";
    std::vector<int> cands = {0, 1, 2, 3};
    for (int a : best_cfg[0])
      for (int b : best_cfg[1])
        for (int c : best_cfg[2]) cands.push_back(sg::split_variant(a, b, c));
    std::vector<std::pair<float, int>> stage1;
    rep += ", \"batched\": {";
    bool firstc = true;
    for (int var : cands) {
      if (sg::batched_max_blocks_per_sm(var) <= 0) continue;
      const float ms = run_batched(var, 0, n_short, true, 1);
      stage1.push_back({ms, var});
      char b[96];
      snprintf(b, sizeof b, "%s\"%d\": %.3f", firstc ? "" : ", ", var, ms);
      firstc = false;
      rep += b;
    }
    rep += "}";
    std::sort(stage1.begin(), stage1.end());
    float best = 1e30f;
    rep += ", \"batched_full\": {";
    const size_t keep = std::min<size_t>(stage1.size(), 12);
    for (size_t k = 0; k < keep; ++k) {
      const int var = stage1[k].second;
      const float ms = n == n_short ? stage1[k].first : run_batched(var, 0, n, true, 3);
      char b[96];
      snprintf(b, sizeof b, "%s\"%d\": %.3f", k ? ", " : "", var, ms);
      rep += b;
      if (ms < best) {
        best = ms;
        chosen[3] = var;
      }
    }
    rep += "}";
    if (chosen[3] >= sg::BATCHED_FUSED_VARIANTS) {
      char b[96];
      snprintf(b, sizeof b, ", \"chosen_configs\": [%d, %d, %d]", sg::split_config(chosen[3], 0), sg::split_config(chosen[3], 1),
               sg::split_config(chosen[3], 2));
      rep += b;
    }
  }
  // plain kernels per curve
  const size_t off[3] = {0, n1, n1 + n2}, cnt[3] = {n1, n2, n3};
  for (int c = 0; c < 3; ++c) {
    float best = 1e30f;
    char b[96];
    snprintf(b, sizeof b, ", \"plain_%d\": {", c);
    rep += b;
    for (int var = 0; var < sg::PLAIN_VARIANTS; ++var) {
      if (sg::plain_max_blocks_per_sm(c, var) <= 0) continue;
      float ms = time_it([&] {
        sg::launch_plain(c, d.p + o_sig + off[c] * 64, d.p + o_msg + off[c] * 32, d.p + o_pk + off[c] * 32, cnt[c], v.gtab[c],
                         d.p + o_out, d.p + o_st, v.d_err, var, st);
      });
      snprintf(b, sizeof b, "%s\"%d\": %.3f", var ? ", " : "", var, ms);
      rep += b;
      if (ms < best) {
        best = ms;
        chosen[c] = var;
      }
    }
    rep += "}";
  }
  char b[160];
  snprintf(b, sizeof b, ", \"chosen\": [%d, %d, %d, %d], \"probe_items\": %zu}", chosen[0], chosen[1], chosen[2], chosen[3], n);
  rep += b;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  sg::fork_streams_destroy(&fork);
  cudaStreamDestroy(st);
  for (int k = 0; k < 4; ++k) {
    int rc = sigops_set_variant(ctx, k, chosen[k]);
    if (rc != SIGOPS_OK) return rc;
  }
  sg::tune_cache_store(v.device, chosen);
  if (report && report_cap) {
    strncpy(report, rep.c_str(), report_cap - 1);
    report[report_cap - 1] = 0;
  }
  return SIGOPS_OK;
}
