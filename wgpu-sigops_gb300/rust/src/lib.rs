//! wgpu_sig_ops on GB300: the batch signature path of the reference crate
//! (src/lib.rs:1-14) with the same module names and public signatures, served
//! by libsigops.so (hand-written sm_103a CUDA) through its C ABI instead of
//! wgpu.  Not compiled here: the build image has no Rust toolchain.
//!
//! Differences a caller can see, all deliberate:
//! - a signature that does not recover gives an empty `Vec<u8>` (the CPU
//!   crates return `Err` for it); the reference fails the whole batch instead;
//! - no power-of-two padding and no 2^22 size cap;
//! - ed25519 rejects a non-canonical S (S >= l), as ed25519-dalek does.

pub mod batch;
pub mod ed25519_eddsa;
pub mod ffi;
pub mod precompute;
pub mod secp256k1_ecdsa;
pub mod secp256r1_ecdsa;

/// A call failed as a whole (src/lib.rs:12-14): a CUDA error, a table that
/// does not match `precompute::*_bases(log_limb_size)`, or a device wait that
/// ran out.
#[derive(Debug, Clone)]
pub struct ShaderFailureError;

/// The library's message for the last failure on this thread.
pub fn last_error() -> String {
    unsafe { std::ffi::CStr::from_ptr(ffi::sigops_last_error()) }.to_string_lossy().into_owned()
}

pub(crate) fn flatten<T, F: Fn(&T) -> Vec<u8>>(items: &[T], bytes: F) -> Vec<u8> {
    let mut v = Vec::new();
    for it in items {
        v.extend_from_slice(&bytes(it));
    }
    v
}

/// ECDSA results: the 64-byte key, or an empty Vec where the status is not OK.
pub(crate) fn keys_or_empty(keys: &[u8], status: &[u8]) -> Vec<Vec<u8>> {
    status
        .iter()
        .enumerate()
        .map(|(i, &s)| if s == ffi::SIGOPS_ST_OK { keys[64 * i..64 * i + 64].to_vec() } else { vec![] })
        .collect()
}
