//! ed25519_eddsa::{ecverify, ecverify_single} (src/ed25519_eddsa.rs:67-324),
//! with ed25519-dalek 2.x `VerifyingKey::verify` semantics per item (a
//! non-canonical S is rejected).  `verify_raw` has no counterpart in the
//! reference: messages of any length instead of 32-byte fuel `Message`s.
use crate::ffi::*;
use crate::{flatten, ShaderFailureError};
use ed25519_dalek::{Signature, VerifyingKey};
use fuel_crypto::Message;

pub async fn ecverify(
    signatures: &Vec<Signature>,
    messages: &Vec<Message>,
    verifying_keys: &Vec<VerifyingKey>,
    table_limbs: &Vec<u32>,
    log_limb_size: u32,
) -> Result<Vec<bool>, ShaderFailureError> {
    let n = signatures.len();
    assert_eq!(n, messages.len());
    assert_eq!(n, verifying_keys.len());
    if n == 0 {
        return Ok(vec![]);
    }
    let sigs = flatten(signatures, |s| s.to_bytes().to_vec());
    let msgs = flatten(messages, |m| m.as_slice().to_vec());
    let pks = flatten(verifying_keys, |k| k.to_bytes().to_vec());
    let mut valid = vec![0u8; n];
    let rc = unsafe {
        sigops_ed25519_ecverify(std::ptr::null_mut(), sigs.as_ptr(), msgs.as_ptr(), pks.as_ptr(), n, table_limbs.as_ptr(),
                                table_limbs.len(), log_limb_size, valid.as_mut_ptr(), std::ptr::null_mut())
    };
    if rc != SIGOPS_OK {
        return Err(ShaderFailureError);
    }
    Ok(valid.into_iter().map(|v| v == 1).collect())
}

pub async fn ecverify_single(
    signatures: &Vec<Signature>,
    messages: &Vec<Message>,
    verifying_keys: &Vec<VerifyingKey>,
    log_limb_size: u32,
) -> Result<Vec<bool>, ShaderFailureError> {
    let n = signatures.len();
    assert_eq!(n, messages.len());
    assert_eq!(n, verifying_keys.len());
    if n == 0 {
        return Ok(vec![]);
    }
    let sigs = flatten(signatures, |s| s.to_bytes().to_vec());
    let msgs = flatten(messages, |m| m.as_slice().to_vec());
    let pks = flatten(verifying_keys, |k| k.to_bytes().to_vec());
    let mut valid = vec![0u8; n];
    let rc = unsafe {
        sigops_ed25519_ecverify_single(std::ptr::null_mut(), sigs.as_ptr(), msgs.as_ptr(), pks.as_ptr(), n, log_limb_size,
                                       valid.as_mut_ptr(), std::ptr::null_mut())
    };
    if rc != SIGOPS_OK {
        return Err(ShaderFailureError);
    }
    Ok(valid.into_iter().map(|v| v == 1).collect())
}

/// Verification over messages of any length (ed25519-dalek
/// `VerifyingKey::verify(&[u8], &Signature)` per item).
pub fn verify_raw(signatures: &[Signature], messages: &[&[u8]], verifying_keys: &[VerifyingKey]) -> Result<Vec<bool>, ShaderFailureError> {
    let n = signatures.len();
    assert_eq!(n, messages.len());
    assert_eq!(n, verifying_keys.len());
    if n == 0 {
        return Ok(vec![]);
    }
    let sigs = flatten(signatures, |s| s.to_bytes().to_vec());
    let pks = flatten(verifying_keys, |k| k.to_bytes().to_vec());
    let mut bytes = Vec::new();
    let mut offsets = Vec::with_capacity(n);
    let mut lens = Vec::with_capacity(n);
    for m in messages {
        offsets.push(bytes.len() as u64);
        lens.push(m.len() as u32);
        bytes.extend_from_slice(m);
    }
    let mut valid = vec![0u8; n];
    let rc = unsafe {
        sigops_ed25519_verify_raw(std::ptr::null_mut(), sigs.as_ptr(), bytes.as_ptr(), bytes.len(), offsets.as_ptr(), lens.as_ptr(),
                                  pks.as_ptr(), n, valid.as_mut_ptr(), std::ptr::null_mut())
    };
    if rc != SIGOPS_OK {
        return Err(ShaderFailureError);
    }
    Ok(valid.into_iter().map(|v| v == 1).collect())
}
