/*
 * sigops.h -- C ABI of the GB300-native batch signature engine.
 *
 * Drop-in boundary for the batch signature path of wgpu_sig_ops
 * (FuelLabs/wgpu-sigops): secp256k1 / secp256r1 ECDSA public-key recovery
 * (`ecrecover`), ed25519 verification (`ecverify`) and the generator-table API
 * `precompute::*_bases(log_limb_size)`.  Every entry point replaces the Rust
 * function cited beside it (paths relative to the reference repository); a
 * Rust crate binds them with one `extern "C"` block and keeps its public
 * signatures.
 *
 * Conventions
 *  - Plain pointers and sizes, caller-owned buffers, no exceptions across the
 *    ABI.  Functions return SIGOPS_OK (0) or a negative SIGOPS_E_* code.
 *  - Byte layouts are the reference's: signatures 64 bytes per item
 *    (ECDSA: r || s big-endian with the recovery parity in bit 7 of byte 32,
 *    fuel-crypto encoding; ed25519: R || S), messages 32 bytes (fuel
 *    `Message`), ed25519 keys 32 bytes (compressed), recovered keys 64 bytes
 *    (x || y big-endian, `PublicKey::as_slice()` / `to_sec1_bytes()[1..65]`).
 *  - Per-item status codes (SIGOPS_ST_*) extend the reference, which reports
 *    only a whole-batch `ShaderFailureError` (src/lib.rs:12-14): an item whose
 *    status is not SIGOPS_ST_OK has a zeroed key (ECDSA) or `false` (ed25519);
 *    the Rust wrapper maps it to an empty `Vec<u8>`, matching the CPU crates'
 *    `Err` for that signature.
 *  - A context owns its CUDA streams, the device-resident generator tables and
 *    staging buffers.  Calls on one context are serialised internally; use
 *    several contexts for concurrency.  `ctx == NULL` selects a process-wide
 *    default context on device 0, created on first use.
 *  - n == 0 returns SIGOPS_OK without touching the GPU (the reference returns
 *    Ok(vec![]), src/secp256k1_ecdsa.rs:71-73).  There is no power-of-two
 *    padding and no 2^22 cap (src/secp256k1_ecdsa.rs:22-44).
 */
#ifndef SIGOPS_H
#define SIGOPS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* return codes */
#define SIGOPS_OK 0
#define SIGOPS_E_INVAL (-22)     /* bad argument (null pointer, unknown curve, bad log_limb_size, misaligned device pointer) */
#define SIGOPS_E_NOMEM (-12)     /* device or pinned host allocation failed */
#define SIGOPS_E_NODEV (-19)     /* no CUDA device / device index out of range */
#define SIGOPS_E_CUDA (-5)       /* CUDA runtime error (see sigops_last_error) */
#define SIGOPS_E_TABLE (-74)     /* table_limbs do not match precompute::*_bases(log_limb_size) */
#define SIGOPS_E_TIMEDOUT (-110) /* a bounded device wait expired (the kernel returned instead of hanging) */
#define SIGOPS_E_BUSY (-16)      /* serving queue full / admission refused */
#define SIGOPS_E_RANGE (-34)     /* batch larger than the fixed capacity of an entry point */
#define SIGOPS_E_CANCELED (-125) /* the serving request was cancelled (sigops_server_cancel) */
#define SIGOPS_ALREADY_DONE 1    /* sigops_server_cancel: the request had finished; its results are in place */

/* curves */
#define SIGOPS_SECP256K1 0
#define SIGOPS_SECP256R1 1
#define SIGOPS_ED25519 2

/* per-item status */
#define SIGOPS_ST_OK 0         /* recovered / verified */
#define SIGOPS_ST_BAD_SCALAR 1 /* ECDSA: r or s outside [1, n-1]; ed25519: S >= l (non-canonical) */
#define SIGOPS_ST_NO_POINT 2   /* ECDSA: r is not the x-coordinate of a curve point; ed25519: key does not decompress */
#define SIGOPS_ST_INFINITY 3   /* ECDSA: the recovered key is the point at infinity */
#define SIGOPS_ST_MISMATCH 4   /* ed25519: [S]B - [k]A does not encode to R */

typedef struct sigops_ctx sigops_ctx;
typedef struct sigops_plan sigops_plan;
typedef struct sigops_server sigops_server;

/* ---------------------------------------------------------------- context */

/* Create a context on `device`.  Builds and uploads the generator tables.
 * Returns NULL on failure (sigops_last_error() says why). */
sigops_ctx* sigops_create(int device);
void sigops_destroy(sigops_ctx* ctx);
/* Message for the last failure on this thread (never NULL). */
const char* sigops_last_error(void);
const char* sigops_strerror(int code);
/* Library version string. */
const char* sigops_version(void);

/* ------------------------------------------------------- generator tables */

/* Number of u32 limbs precompute::*_bases(log_limb_size) returns for `curve`
 * (16 points x {2,3} coordinates x ceil(256/L) limbs), or SIGOPS_E_INVAL.
 * log_limb_size must be in [11, 15], the range the reference's Montgomery
 * shaders support (src/wgsl/mont.wgsl:12,37). */
long sigops_bases_len(int curve, uint32_t log_limb_size);

/* precompute::secp256k1_bases / secp256r1_bases / ed25519_bases
 * (src/precompute.rs:36-69): writes the table, bit-identical to the reference,
 * into out[0 .. cap) and returns its length (or a negative code).  CPU only;
 * needs no GPU. */
long sigops_bases(int curve, uint32_t log_limb_size, uint32_t* out, size_t cap);

/* SIGOPS_OK if table_limbs equals precompute::*_bases(log_limb_size), else
 * SIGOPS_E_TABLE (or SIGOPS_E_INVAL for a bad log_limb_size).  CPU only. */
int sigops_check_table(int curve, const uint32_t* table_limbs, size_t table_len, uint32_t log_limb_size);

/* --------------------------------------------- drop-in calls, host buffers */

/* secp256k1_ecdsa::ecrecover (src/secp256k1_ecdsa.rs:61-213).
 * sigs: n*64 bytes, msgs: n*32 bytes, out_pubkeys: n*64 bytes,
 * out_status: n bytes (may be NULL).  table_limbs/table_len/log_limb_size are
 * validated against precompute::secp256k1_bases (SIGOPS_E_TABLE on mismatch);
 * the kernels use their own wider device-resident tables. */
int sigops_secp256k1_ecrecover(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* table_limbs,
                               size_t table_len, uint32_t log_limb_size, uint8_t* out_pubkeys, uint8_t* out_status);

/* secp256k1_ecdsa::ecrecover_single_shader (src/secp256k1_ecdsa.rs:215-274). */
int sigops_secp256k1_ecrecover_single_shader(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, size_t n,
                                             uint32_t log_limb_size, uint8_t* out_pubkeys, uint8_t* out_status);

/* secp256r1_ecdsa::ecrecover (src/secp256r1_ecdsa.rs; signatures are fuel
 * Bytes64 with the same encoding). */
int sigops_secp256r1_ecrecover(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* table_limbs,
                               size_t table_len, uint32_t log_limb_size, uint8_t* out_pubkeys, uint8_t* out_status);

/* secp256r1_ecdsa::ecrecover_single_shader (src/secp256r1_ecdsa.rs). */
int sigops_secp256r1_ecrecover_single_shader(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, size_t n,
                                             uint32_t log_limb_size, uint8_t* out_pubkeys, uint8_t* out_status);

/* ed25519_eddsa::ecverify (src/ed25519_eddsa.rs:67-257).
 * sigs: n*64 (R || S), msgs: n*32, pks: n*32 (VerifyingKey::to_bytes()),
 * out_valid: n bytes of 0/1, out_status: n bytes (may be NULL). */
int sigops_ed25519_ecverify(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n,
                            const uint32_t* table_limbs, size_t table_len, uint32_t log_limb_size, uint8_t* out_valid,
                            uint8_t* out_status);

/* ed25519_eddsa::ecverify_single (src/ed25519_eddsa.rs:259-324). */
int sigops_ed25519_ecverify_single(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n,
                                   uint32_t log_limb_size, uint8_t* out_valid, uint8_t* out_status);

/* ed25519 verification of messages of any length (ed25519-dalek
 * VerifyingKey::verify(&[u8], &Signature) semantics, per item as
 * sigops_ed25519_ecverify).  No counterpart in the reference, whose API
 * passes 32-byte fuel messages (src/ed25519_eddsa.rs:67-74).  Message i is
 * msgs[msg_offsets[i] .. msg_offsets[i] + msg_lens[i]); every message must lie
 * within the msgs_bytes bytes of msgs (else SIGOPS_E_INVAL).  The challenge
 * SHA-512(R || A || M) runs ceil((81 + len) / 128) blocks on the GPU. */
int sigops_ed25519_verify_raw(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, size_t msgs_bytes, const uint64_t* msg_offsets,
                              const uint32_t* msg_lens, const uint8_t* pks, size_t n, uint8_t* out_valid, uint8_t* out_status);

/* ------------------------------------------ device-resident plain kernels */

/* One plain (one signature per thread) kernel over device buffers on `stream`
 * (a cudaStream_t; NULL = the context's stream).  No host synchronisation.
 * Pointers must be 16-byte aligned.  ECDSA: d_out receives n*64 key bytes;
 * ed25519: d_out receives n validity bytes and d_pks is required.
 * Device-side failures (a bounded wait that expired) are reported by the next
 * sigops_sync().  Equivalent of one reference dispatch
 * (src/gpu.rs:88-104) without its per-call device creation. */
int sigops_plain_device(sigops_ctx* ctx, int curve, const uint8_t* d_sigs, const uint8_t* d_msgs, const uint8_t* d_pks, size_t n,
                        uint8_t* d_out, uint8_t* d_status, void* stream);

/* ----------------------------------------- batched mixed-curve engine */

/* Verify a batch that mixes the three curves in one call of the batched engine
 * (classify, then the context's launch variant).  No counterpart in the
 * reference, which runs one curve per call with
 * power-of-two padding (src/secp256k1_ecdsa.rs:25-44); per-item semantics are
 * those of the per-curve calls above.
 * curves: n tags (SIGOPS_SECP256K1 / SECP256R1 / ED25519); sigs n*64; msgs
 * n*32; pks n*32 (read for ed25519 items only); out n*64 (ECDSA: key bytes;
 * ed25519: byte 0 = valid, rest zero); out_status n (may be NULL).  When all
 * buffers are page-locked and n >= 131072, the call runs as two halves on
 * two streams (the first at the highest priority), so that copies overlap
 * the other half's kernels.  n < 2^32 (the index lists hold 32-bit item
 * indices), else SIGOPS_E_RANGE. */
int sigops_verify_mixed(sigops_ctx* ctx, const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n,
                        uint8_t* out, uint8_t* out_status);

/* Same over device buffers (16-byte aligned) on `stream`; no host sync.
 * Uses context-owned scratch sized by sigops_reserve (grown on demand, which
 * allocates: reserve first when capturing into a CUDA graph). */
int sigops_verify_mixed_device(sigops_ctx* ctx, const uint8_t* d_curves, const uint8_t* d_sigs, const uint8_t* d_msgs, const uint8_t* d_pks,
                               size_t n, uint8_t* d_out, uint8_t* d_status, void* stream);

/* Allocation-free form of sigops_verify_mixed_device.  No counterpart in the
 * reference.  It exists for callers that cannot allocate device memory per
 * call: processes whose GPU memory belongs to another allocator (a
 * framework's caching allocator, or a budget reserved once at start-up) and
 * latency-critical verifier threads that cannot absorb cudaMalloc's implicit
 * device synchronisation.  It needs no context and calls no cudaMalloc or
 * cudaFree: its scratch (counters and per-curve index lists), the generator
 * tables and its error word are file-scope static device arrays, which every
 * GPU that loads the library holds until the process exits (about 10 MiB,
 * mostly the generator tables, separate from any context's tables).
 * Limit: n <= SIGOPS_NOALLOC_MAX_ITEMS, else SIGOPS_E_RANGE.  Buffers and
 * results as sigops_verify_mixed_device: device pointers (16-byte aligned)
 * on the current device, work queued on `stream`, no host synchronisation.
 * The first call on each device does a one-time set-up (symbol addresses,
 * table upload, one device synchronisation): make that first call before any
 * stream capture.  Every call shares the static scratch and clears the
 * counters it uses, so calls whose work overlaps on the GPU race: serialise
 * them. */
#define SIGOPS_NOALLOC_MAX_ITEMS 65536
int sigops_verify_mixed_noalloc(const uint8_t* d_curves, const uint8_t* d_sigs, const uint8_t* d_msgs, const uint8_t* d_pks, size_t n,
                                uint8_t* d_out, uint8_t* d_status, void* stream);

/* Device-side errors of the allocation-free calls on the current device: reads
 * the static error word after the work queued on `stream`, waits for that
 * read, and clears the word.  SIGOPS_OK, or SIGOPS_E_TIMEDOUT when a bounded
 * device wait of an earlier call expired.  Allocates nothing.  No
 * counterpart in the reference. */
int sigops_noalloc_status(void* stream);

/* Size the context's batched-engine scratch for batches of up to n items. */
int sigops_reserve(sigops_ctx* ctx, size_t n);

/* A CUDA graph of one batched step over fixed device buffers: the scratch
 * reset, the classify kernel and the batched engine's kernels for the
 * context's launch variant (for the single-curve variants three kernels on
 * parallel graph branches), replayed by sigops_mixed_plan_launch.  The plan
 * uses the context's scratch: do not run two plans or mixed calls of one
 * context concurrently. */
int sigops_mixed_plan_create(sigops_ctx* ctx, const uint8_t* d_curves, const uint8_t* d_sigs, const uint8_t* d_msgs, const uint8_t* d_pks,
                             size_t n, uint8_t* d_out, uint8_t* d_status, sigops_plan** plan);
int sigops_mixed_plan_launch(sigops_plan* plan, void* stream);
void sigops_mixed_plan_destroy(sigops_plan* plan);

/* Launch-shape variants (the autotuner's search space).  kernel 0..2: the
 * plain kernel of SIGOPS_SECP256K1 / SECP256R1 / ED25519, variant 0 = one
 * 256-thread block per SM, 1 = two (register budget 128), 2 = 128 threads x 3
 * blocks (budget 170); kernel 3: the batched engine, variants 0..3 = the fused
 * mixed-curve kernel: 0 = persistent, 256 threads x 1 block per SM; 1 = one
 * 32-item tile per warp, 256 threads; 2 = one tile per warp, 128 threads x 3
 * blocks (170 registers); 3 = one tile per warp, 256 threads x 2 blocks (128
 * registers); variants 4 + a + 4 b + 16 c (4..67) = three single-curve
 * kernels run side by side on forked streams, secp256k1 at occupancy level a,
 * P-256 at b, ed25519 at c (level 0 = 256 threads x 1 block per SM, 1 = 128
 * threads x 3 blocks, register budget 170; 2 = 256 x 2, budget 128; 3 = 64
 * threads, at most 144 registers: 7 blocks per SM).
 * sigops_get_variant also reports the grid and block used. */
int sigops_set_variant(sigops_ctx* ctx, int kernel, int variant);
int sigops_get_variant(sigops_ctx* ctx, int kernel, int* variant, int* grid, int* block);

/* Autotuner: signs a probe batch (probe_items, 0 = 16 waves of the device) with
 * the 40/30/30 curve mix on the device, times every variant of each plain
 * kernel (best of three after a warm-up) and of the batched engine (all
 * variants once on an 8-wave prefix, then the twelve fastest on the whole probe,
 * best of three), and selects the fastest.  The batched ranking depends on the
 * batch size: pass the size of the batches that will run.  report (may be
 * NULL) receives a JSON summary of the timings.
 * When SIGOPS_TUNE_CACHE names a file, the choice is stored there per device
 * model and sigops_create applies it. */
int sigops_autotune(sigops_ctx* ctx, size_t probe_items, char* report, size_t report_cap);

/* ------------------------------------------------------- serving loop */

/* A continuous-batching server over one context (no counterpart in the
 * reference).  Its queues live with the device: submit copies a request's
 * items into a pinned, mapped request ring and cuts them into 32-item
 * single-curve tiles; one persistent kernel (launched cooperatively, every
 * block resident) copies published tiles into a device-resident tile ring and
 * works them off, results going straight to a pinned output ring; a host
 * dispatcher thread copies each finished request's results to the caller's
 * buffers and relaunches the kernel after it closes (20 ms idle, or 2 s of
 * life).  Requests that arrive while others run become tiles behind them: no
 * launch, copy or host round trip per request.  Every device-side wait is
 * bounded; an expired one fails the requests in flight (SIGOPS_E_TIMEDOUT)
 * instead of hanging them.  While the kernel runs it holds every SM it is
 * resident on: other work of the context waits for its idle close.
 * slot_items: the largest request (0 = 16,384); slots x slot_items: items in
 * flight at most (slots <= 0 selects 32), within hbm_fraction (default 0.25)
 * of the device memory free at creation.  Returns NULL on failure. */
sigops_server* sigops_server_create(sigops_ctx* ctx, int slots, size_t slot_items, double hbm_fraction);
/* Stops the kernel and the server's threads and frees everything; no other
 * thread may be inside a call on the server.  Requests still in flight are
 * dropped (their buffers are not written after this returns). */
void sigops_server_destroy(sigops_server* server);
size_t sigops_server_slot_items(sigops_server* server);
/* Shape of the persistent kernel: 0 = 256-thread blocks, one per SM (default);
 * 1 = 128 x 3 per SM (170 registers); 2 = 256 x 2 (128 registers).  Applies
 * from the next launch of the kernel, and ends an adaptive choice.  No
 * counterpart in the reference. */
int sigops_server_set_variant(sigops_server* server, int variant);

/* Adaptive shape: each launch of the persistent kernel takes high_shape while
 * the arrival rate (items accepted by submit per second, a moving average of
 * 10 ms samples with weight 1/4: about 40 ms to follow a step) is at least
 * switch_items_per_s, and low_shape once it falls below 80% of it.  A running launch of the other shape is asked to close (after
 * every tile already published) once it has run 20 ms.  Typically
 * low_shape has the fewer warps per SM (lower latency) and high_shape the
 * higher saturation.  SIGOPS_E_INVAL for a bad shape or a rate <= 0.  No
 * counterpart in the reference. */
int sigops_server_set_adaptive(sigops_server* server, int low_shape, int high_shape, double switch_items_per_s);

/* The shape of the running (or last) launch, the number of shape switches
 * the adaptive choice asked for, and the arrival-rate estimate (items/s).
 * Any pointer may be NULL. */
int sigops_server_shape_stats(sigops_server* server, int* shape, uint64_t* switches, double* items_per_s);

/* Queue one request of n items.  curves: n tags, or NULL with uniform_curve
 * set for a single-curve request; pks may be NULL for ECDSA-only requests.
 * The inputs are copied before the call returns; out (n*64 bytes, mixed
 * record layout) and status (n bytes, may be NULL) must stay valid until
 * sigops_server_wait or sigops_server_cancel returns for the handle.
 * Admission, checked now: SIGOPS_E_RANGE if n exceeds slot_items;
 * SIGOPS_E_BUSY if the request rings have no room for it or the device's free
 * memory is below its floor (1% of the device, at least 256 MiB; re-read every
 * 100 ms); SIGOPS_E_CUDA if the server can no longer run requests. */
int sigops_server_submit(sigops_server* server, const uint8_t* curves, int uniform_curve, const uint8_t* sigs, const uint8_t* msgs,
                         const uint8_t* pks, size_t n, uint8_t* out, uint8_t* status, uint64_t* handle);

/* Wait for a request (timeout_ms < 0: no limit).  SIGOPS_OK when its results
 * are in place (latency_ms: submit to results, may be NULL) and the handle is
 * released; SIGOPS_E_TIMEDOUT if still running (or the server's dispatcher
 * stopped); SIGOPS_E_CANCELED if it was cancelled; SIGOPS_E_INVAL for an
 * unknown handle. */
int sigops_server_wait(sigops_server* server, uint64_t handle, int timeout_ms, double* latency_ms);

/* Withdraw a request: SIGOPS_OK when its results will not be written (the
 * handle is released and the caller's out / status buffers may be freed at
 * once; the device still works the items off and drops them);
 * SIGOPS_ALREADY_DONE when it had finished (its results are in place; wait
 * releases the handle); SIGOPS_E_INVAL for an unknown handle.  No
 * counterpart in the reference. */
int sigops_server_cancel(sigops_server* server, uint64_t handle);

int sigops_server_stats(sigops_server* server, uint64_t* launches, uint64_t* requests_done, uint64_t* items_done, size_t* queued_items);

/* Counters of the persistent kernel since the server was created: tiles and
 * items verified, the time its warps spent working on tiles and looking for
 * one (seconds, summed over warps; work / (work + idle) is how busy the GPU
 * was while the kernel ran), and how often an SM changed the curve it works
 * on.  Any pointer may be NULL.  No counterpart in the reference. */
int sigops_server_kernel_stats(sigops_server* server, uint64_t* tiles, uint64_t* items, double* work_s, double* idle_s,
                               uint64_t* sm_moves);

/* The dispatcher thread: iterations so far, the longest time between two
 * iterations with requests in flight and the longest driver call it made
 * (kernel relaunch, exit check), both since the previous call (ms; waiting
 * threads also collect completions, so a late dispatcher delays relaunches
 * rather than results).  No counterpart in the reference. */
int sigops_server_dispatch_stats(sigops_server* server, uint64_t* iterations, double* max_gap_ms, double* max_driver_ms);

/* Open-loop load generator: request i covers pool items
 * [offset[i], offset[i] + count[i]) and is submitted arrival_s[i] seconds after
 * the start (non-decreasing) by one of four client threads (request i by
 * thread i mod 4), while the calling thread waits for the requests in order;
 * outputs go to the same item positions of out / status.  Fills
 * latency_ms[i] (-1 when refused) and the wall time. */
int sigops_server_run_load(sigops_server* server, const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks,
                           const uint64_t* offset, const uint32_t* count, const double* arrival_s, size_t nreq, uint8_t* out,
                           uint8_t* status, double* latency_ms, double* wall_s);

/* Failure injection for tests, on the host (no device fault): fault 1 makes
 * the server's dispatcher thread stop at its next iteration, as if it had
 * died; waits then return SIGOPS_E_TIMEDOUT and submits SIGOPS_E_CUDA, and
 * sigops_server_destroy still cleans up.  No counterpart in the reference. */
int sigops_server_test_fault(sigops_server* server, int fault);

/* Failure injection for tests, on the host: the next `count` device or pinned
 * host allocations made by the library fail as if out of memory (0 clears).
 * Returns the previous count.  No counterpart in the reference. */
int sigops_test_fail_allocations(int count);

/* ------------------------------------------- synthetic workload signing */

/* Sign on the device to generate benchmark / test inputs (no counterpart on
 * the reference's path, whose tests sign on the CPU with fuel-crypto / p256 /
 * ed25519-dalek).  ECDSA: secret and nonce 32 bytes big-endian per item;
 * writes fuel-encoded low-s signatures (n*64), public keys (n*64) and a status
 * byte (0 ok, 1 the secret/nonce pair cannot sign).  ed25519: RFC 8032 from
 * 32-byte seeds; writes signatures (n*64) and keys (n*32). */
int sigops_workload_sign_ecdsa(sigops_ctx* ctx, int curve, const uint8_t* d_secrets, const uint8_t* d_nonces, const uint8_t* d_msgs, size_t n,
                               uint8_t* d_sigs, uint8_t* d_pubkeys, uint8_t* d_status, void* stream);
int sigops_workload_sign_ed25519(sigops_ctx* ctx, const uint8_t* d_seeds, const uint8_t* d_msgs, size_t n, uint8_t* d_sigs, uint8_t* d_pks,
                                 void* stream);

/* Wait for the context's stream and report device-side errors since the last
 * call (SIGOPS_E_TIMEDOUT if a bounded wait expired). */
int sigops_sync(sigops_ctx* ctx);

/* ------------------------------------------------------------ diagnostics */

/* Measured 32-bit integer multiply-add throughput of this device (IMAD per
 * second), from a dependency-free mad.lo probe timed with CUDA events. */
int sigops_probe_imad(sigops_ctx* ctx, double* imad_per_second);

/* Measured multiply-instruction throughput (per second) of one instruction
 * form: 0 = mad.lo.u32, 1 = mad.hi.u32, 2 = carry-chain rows alternating
 * mad.lo.cc / madc.hi.cc (the form of the field multiplications), 3 =
 * mad.wide.u32.  No counterpart in the reference; the roofline denominator. */
int sigops_probe_mul(sigops_ctx* ctx, int form, double* per_second);

/* Threads per signature, measured: secp256k1 recovery of the n signatures in
 * device buffers d_sigs / d_msgs by one thread per signature (lanes = 1, the
 * plain path) or by a lane pair per signature (lanes = 2: the GLV halves of
 * both scalars on the two lanes, partial sums combined by shuffles), in
 * blocks of `block` threads (a multiple of 32 up to 256; 0 = 256).  Results
 * go to d_out (n x 64) / d_status (n); *ms = the kernel's time, CUDA events,
 * after one warm-up launch.  Test and measurement only.  No counterpart in the
 * reference. */
int sigops_probe_k1_lanes(sigops_ctx* ctx, int lanes, int block, const uint8_t* d_sigs, const uint8_t* d_msgs, size_t n, uint8_t* d_out,
                          uint8_t* d_status, float* ms);

/* Warp phases, measured: secp256k1 recovery of the n signatures in device
 * buffers d_sigs / d_msgs (one thread per signature) by persistent warps, one
 * 256-thread block per SM, each warp taking 32 items at a time: free-running
 * (sync = 0, as the serving kernel's warps) or with a block's warps starting
 * every group together (sync = 1, as a plain kernel's block).  Results go to
 * d_out (n x 64) / d_status (n); d_times (2 ceil(n / 32) words) receives the
 * global-timer start and end of each group of 32 items (ns); *ms = the
 * kernel's time, CUDA events.  Test and measurement only.  No counterpart in
 * the reference. */
int sigops_probe_phase(sigops_ctx* ctx, int sync, const uint8_t* d_sigs, const uint8_t* d_msgs, size_t n, uint8_t* d_out,
                       uint8_t* d_status, uint64_t* d_times, float* ms);

/* Number of SMs and the plain kernels' grid (blocks) for `curve`. */
int sigops_device_info(sigops_ctx* ctx, int* num_sms, int* plain_grid_k1, int* plain_grid_r1, int* plain_grid_ed);

/* Arithmetic self-test hooks (run the kernels' field / hash code on the
 * device): field 0..5 = secp256k1 p, P-256 p, 2^255-19, secp256k1 n,
 * P-256 n, l; op 0 mul, 1 add, 2 sub, 3 inverse, 4 square-root candidate /
 * (p-5)/8 power, 5 full 512-bit product.  a, b, out: host arrays of n 32-byte
 * little-endian integers (out: 2n entries). */
int sigops_test_field(sigops_ctx* ctx, int field, int op, const uint8_t* a, const uint8_t* b, uint8_t* out, size_t n);
/* SHA-512 of n 96-byte inputs (R || A || M preimages); out n*64 bytes. */
int sigops_test_sha512(sigops_ctx* ctx, const uint8_t* in, uint8_t* out, size_t n);

/* Exercises the expiry of the kernels' bounded waits without any fault: a
 * one-block kernel waits, at most max_polls polls (1..65536), on an mbarrier
 * that nothing arrives on.  Returns SIGOPS_E_TIMEDOUT (the device error word
 * is read and cleared, and the context stays usable).  No counterpart in the
 * reference. */
int sigops_test_wait_expiry(sigops_ctx* ctx, uint32_t max_polls);

#ifdef __cplusplus
}
#endif

#endif /* SIGOPS_H */
