//! secp256k1_ecdsa::{ecrecover, ecrecover_single_shader}
//! (src/secp256k1_ecdsa.rs:61-274).  Signatures are fuel-crypto 64-byte
//! encodings (recovery parity in bit 7 of byte 32); results are 64-byte x || y
//! keys (`PublicKey::as_slice()`), empty where a signature does not recover.
use crate::ffi::*;
use crate::{flatten, keys_or_empty, ShaderFailureError};
use fuel_crypto::{Message, Signature};

pub async fn ecrecover(
    signatures: &Vec<Signature>,
    messages: &Vec<Message>,
    table_limbs: &Vec<u32>,
    log_limb_size: u32,
) -> Result<Vec<Vec<u8>>, ShaderFailureError> {
    assert_eq!(signatures.len(), messages.len()); // src/secp256k1_ecdsa.rs:21
    let n = signatures.len();
    if n == 0 {
        return Ok(vec![]);
    }
    let sigs = flatten(signatures, |s| s.as_slice().to_vec());
    let msgs = flatten(messages, |m| m.as_slice().to_vec());
    let mut keys = vec![0u8; 64 * n];
    let mut status = vec![0u8; n];
    let rc = unsafe {
        sigops_secp256k1_ecrecover(std::ptr::null_mut(), sigs.as_ptr(), msgs.as_ptr(), n, table_limbs.as_ptr(), table_limbs.len(),
                                   log_limb_size, keys.as_mut_ptr(), status.as_mut_ptr())
    };
    if rc != SIGOPS_OK {
        return Err(ShaderFailureError);
    }
    Ok(keys_or_empty(&keys, &status))
}

pub async fn ecrecover_single_shader(
    signatures: &Vec<Signature>,
    messages: &Vec<Message>,
    log_limb_size: u32,
) -> Result<Vec<Vec<u8>>, ShaderFailureError> {
    assert_eq!(signatures.len(), messages.len());
    let n = signatures.len();
    if n == 0 {
        return Ok(vec![]);
    }
    let sigs = flatten(signatures, |s| s.as_slice().to_vec());
    let msgs = flatten(messages, |m| m.as_slice().to_vec());
    let mut keys = vec![0u8; 64 * n];
    let mut status = vec![0u8; n];
    let rc = unsafe {
        sigops_secp256k1_ecrecover_single_shader(std::ptr::null_mut(), sigs.as_ptr(), msgs.as_ptr(), n, log_limb_size, keys.as_mut_ptr(),
                                                 status.as_mut_ptr())
    };
    if rc != SIGOPS_OK {
        return Err(ShaderFailureError);
    }
    Ok(keys_or_empty(&keys, &status))
}
