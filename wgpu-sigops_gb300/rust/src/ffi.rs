//! Raw declarations of libsigops.so's C ABI (include/sigops.h), one per
//! exported function.  Not compiled here: the build image has no Rust
//! toolchain; tests/test_abi.py checks that this file declares every function
//! the header declares.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_long, c_void};

#[repr(C)]
pub struct SigopsCtx {
    _p: [u8; 0],
}
#[repr(C)]
pub struct SigopsPlan {
    _p: [u8; 0],
}
#[repr(C)]
pub struct SigopsServer {
    _p: [u8; 0],
}

pub const SIGOPS_OK: c_int = 0;
pub const SIGOPS_E_INVAL: c_int = -22;
pub const SIGOPS_E_NOMEM: c_int = -12;
pub const SIGOPS_E_NODEV: c_int = -19;
pub const SIGOPS_E_CUDA: c_int = -5;
pub const SIGOPS_E_TABLE: c_int = -74;
pub const SIGOPS_E_TIMEDOUT: c_int = -110;
pub const SIGOPS_E_BUSY: c_int = -16;
pub const SIGOPS_E_RANGE: c_int = -34;
pub const SIGOPS_E_CANCELED: c_int = -125;
pub const SIGOPS_ALREADY_DONE: c_int = 1;

pub const SIGOPS_SECP256K1: c_int = 0;
pub const SIGOPS_SECP256R1: c_int = 1;
pub const SIGOPS_ED25519: c_int = 2;

pub const SIGOPS_ST_OK: u8 = 0;
pub const SIGOPS_ST_BAD_SCALAR: u8 = 1;
pub const SIGOPS_ST_NO_POINT: u8 = 2;
pub const SIGOPS_ST_INFINITY: u8 = 3;
pub const SIGOPS_ST_MISMATCH: u8 = 4;

pub const SIGOPS_NOALLOC_MAX_ITEMS: usize = 65536;

extern "C" {
    // context
    pub fn sigops_create(device: c_int) -> *mut SigopsCtx;
    pub fn sigops_destroy(ctx: *mut SigopsCtx);
    pub fn sigops_last_error() -> *const c_char;
    pub fn sigops_strerror(code: c_int) -> *const c_char;
    pub fn sigops_version() -> *const c_char;

    // generator tables (precompute::*_bases)
    pub fn sigops_bases_len(curve: c_int, log_limb_size: u32) -> c_long;
    pub fn sigops_bases(curve: c_int, log_limb_size: u32, out: *mut u32, cap: usize) -> c_long;
    pub fn sigops_check_table(curve: c_int, table_limbs: *const u32, table_len: usize, log_limb_size: u32) -> c_int;

    // drop-in calls over host buffers
    pub fn sigops_secp256k1_ecrecover(ctx: *mut SigopsCtx, sigs: *const u8, msgs: *const u8, n: usize, table_limbs: *const u32,
                                      table_len: usize, log_limb_size: u32, out_pubkeys: *mut u8, out_status: *mut u8) -> c_int;
    pub fn sigops_secp256k1_ecrecover_single_shader(ctx: *mut SigopsCtx, sigs: *const u8, msgs: *const u8, n: usize,
                                                    log_limb_size: u32, out_pubkeys: *mut u8, out_status: *mut u8) -> c_int;
    pub fn sigops_secp256r1_ecrecover(ctx: *mut SigopsCtx, sigs: *const u8, msgs: *const u8, n: usize, table_limbs: *const u32,
                                      table_len: usize, log_limb_size: u32, out_pubkeys: *mut u8, out_status: *mut u8) -> c_int;
    pub fn sigops_secp256r1_ecrecover_single_shader(ctx: *mut SigopsCtx, sigs: *const u8, msgs: *const u8, n: usize,
                                                    log_limb_size: u32, out_pubkeys: *mut u8, out_status: *mut u8) -> c_int;
    pub fn sigops_ed25519_ecverify(ctx: *mut SigopsCtx, sigs: *const u8, msgs: *const u8, pks: *const u8, n: usize,
                                   table_limbs: *const u32, table_len: usize, log_limb_size: u32, out_valid: *mut u8,
                                   out_status: *mut u8) -> c_int;
    pub fn sigops_ed25519_ecverify_single(ctx: *mut SigopsCtx, sigs: *const u8, msgs: *const u8, pks: *const u8, n: usize,
                                          log_limb_size: u32, out_valid: *mut u8, out_status: *mut u8) -> c_int;
    pub fn sigops_ed25519_verify_raw(ctx: *mut SigopsCtx, sigs: *const u8, msgs: *const u8, msgs_bytes: usize, msg_offsets: *const u64,
                                     msg_lens: *const u32, pks: *const u8, n: usize, out_valid: *mut u8, out_status: *mut u8) -> c_int;

    // device-resident plain kernels
    pub fn sigops_plain_device(ctx: *mut SigopsCtx, curve: c_int, d_sigs: *const u8, d_msgs: *const u8, d_pks: *const u8, n: usize,
                               d_out: *mut u8, d_status: *mut u8, stream: *mut c_void) -> c_int;

    // batched mixed-curve engine
    pub fn sigops_verify_mixed(ctx: *mut SigopsCtx, curves: *const u8, sigs: *const u8, msgs: *const u8, pks: *const u8, n: usize,
                               out: *mut u8, out_status: *mut u8) -> c_int;
    pub fn sigops_verify_mixed_device(ctx: *mut SigopsCtx, d_curves: *const u8, d_sigs: *const u8, d_msgs: *const u8, d_pks: *const u8,
                                      n: usize, d_out: *mut u8, d_status: *mut u8, stream: *mut c_void) -> c_int;
    pub fn sigops_verify_mixed_noalloc(d_curves: *const u8, d_sigs: *const u8, d_msgs: *const u8, d_pks: *const u8, n: usize,
                                       d_out: *mut u8, d_status: *mut u8, stream: *mut c_void) -> c_int;
    pub fn sigops_noalloc_status(stream: *mut c_void) -> c_int;
    pub fn sigops_reserve(ctx: *mut SigopsCtx, n: usize) -> c_int;
    pub fn sigops_mixed_plan_create(ctx: *mut SigopsCtx, d_curves: *const u8, d_sigs: *const u8, d_msgs: *const u8, d_pks: *const u8,
                                    n: usize, d_out: *mut u8, d_status: *mut u8, plan: *mut *mut SigopsPlan) -> c_int;
    pub fn sigops_mixed_plan_launch(plan: *mut SigopsPlan, stream: *mut c_void) -> c_int;
    pub fn sigops_mixed_plan_destroy(plan: *mut SigopsPlan);
    pub fn sigops_set_variant(ctx: *mut SigopsCtx, kernel: c_int, variant: c_int) -> c_int;
    pub fn sigops_get_variant(ctx: *mut SigopsCtx, kernel: c_int, variant: *mut c_int, grid: *mut c_int, block: *mut c_int) -> c_int;
    pub fn sigops_autotune(ctx: *mut SigopsCtx, probe_items: usize, report: *mut c_char, report_cap: usize) -> c_int;

    // serving loop
    pub fn sigops_server_create(ctx: *mut SigopsCtx, slots: c_int, slot_items: usize, hbm_fraction: f64) -> *mut SigopsServer;
    pub fn sigops_server_destroy(server: *mut SigopsServer);
    pub fn sigops_server_slot_items(server: *mut SigopsServer) -> usize;
    pub fn sigops_server_set_variant(server: *mut SigopsServer, variant: c_int) -> c_int;
    pub fn sigops_server_set_adaptive(server: *mut SigopsServer, low_shape: c_int, high_shape: c_int, switch_items_per_s: f64) -> c_int;
    pub fn sigops_server_shape_stats(server: *mut SigopsServer, shape: *mut c_int, switches: *mut u64, items_per_s: *mut f64) -> c_int;
    pub fn sigops_server_submit(server: *mut SigopsServer, curves: *const u8, uniform_curve: c_int, sigs: *const u8, msgs: *const u8,
                                pks: *const u8, n: usize, out: *mut u8, status: *mut u8, handle: *mut u64) -> c_int;
    pub fn sigops_server_wait(server: *mut SigopsServer, handle: u64, timeout_ms: c_int, latency_ms: *mut f64) -> c_int;
    pub fn sigops_server_cancel(server: *mut SigopsServer, handle: u64) -> c_int;
    pub fn sigops_server_dispatch_stats(server: *mut SigopsServer, iterations: *mut u64, max_gap_ms: *mut f64,
        max_driver_ms: *mut f64) -> c_int;
    pub fn sigops_server_kernel_stats(server: *mut SigopsServer, tiles: *mut u64, items: *mut u64, work_s: *mut f64,
        idle_s: *mut f64, sm_moves: *mut u64) -> c_int;
    pub fn sigops_server_test_fault(server: *mut SigopsServer, fault: c_int) -> c_int;
    pub fn sigops_server_stats(server: *mut SigopsServer, launches: *mut u64, requests_done: *mut u64, items_done: *mut u64,
                               queued_items: *mut usize) -> c_int;
    pub fn sigops_server_run_load(server: *mut SigopsServer, curves: *const u8, sigs: *const u8, msgs: *const u8, pks: *const u8,
                                  offset: *const u64, count: *const u32, arrival_s: *const f64, nreq: usize, out: *mut u8,
                                  status: *mut u8, latency_ms: *mut f64, wall_s: *mut f64) -> c_int;

    // synthetic workload signing
    pub fn sigops_workload_sign_ecdsa(ctx: *mut SigopsCtx, curve: c_int, d_secrets: *const u8, d_nonces: *const u8, d_msgs: *const u8,
                                      n: usize, d_sigs: *mut u8, d_pubkeys: *mut u8, d_status: *mut u8, stream: *mut c_void) -> c_int;
    pub fn sigops_workload_sign_ed25519(ctx: *mut SigopsCtx, d_seeds: *const u8, d_msgs: *const u8, n: usize, d_sigs: *mut u8,
                                        d_pks: *mut u8, stream: *mut c_void) -> c_int;
    pub fn sigops_sync(ctx: *mut SigopsCtx) -> c_int;

    // diagnostics
    pub fn sigops_probe_imad(ctx: *mut SigopsCtx, imad_per_second: *mut f64) -> c_int;
    pub fn sigops_probe_mul(ctx: *mut SigopsCtx, form: c_int, per_second: *mut f64) -> c_int;
    pub fn sigops_probe_k1_lanes(ctx: *mut SigopsCtx, lanes: c_int, block: c_int, d_sigs: *const u8, d_msgs: *const u8, n: usize,
        d_out: *mut u8, d_status: *mut u8, ms: *mut f32) -> c_int;
    pub fn sigops_probe_phase(ctx: *mut SigopsCtx, sync: c_int, d_sigs: *const u8, d_msgs: *const u8, n: usize, d_out: *mut u8,
        d_status: *mut u8, d_times: *mut u64, ms: *mut f32) -> c_int;
    pub fn sigops_device_info(ctx: *mut SigopsCtx, num_sms: *mut c_int, plain_grid_k1: *mut c_int, plain_grid_r1: *mut c_int,
                              plain_grid_ed: *mut c_int) -> c_int;
    pub fn sigops_test_field(ctx: *mut SigopsCtx, field: c_int, op: c_int, a: *const u8, b: *const u8, out: *mut u8, n: usize) -> c_int;
    pub fn sigops_test_sha512(ctx: *mut SigopsCtx, input: *const u8, out: *mut u8, n: usize) -> c_int;
    pub fn sigops_test_wait_expiry(ctx: *mut SigopsCtx, max_polls: u32) -> c_int;
    pub fn sigops_test_fail_allocations(count: c_int) -> c_int;
}
