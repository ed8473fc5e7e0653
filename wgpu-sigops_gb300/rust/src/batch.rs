//! The batched mixed-curve engine: one call over a batch that mixes
//! secp256k1 recovery, P-256 recovery and ed25519 verification.  No
//! counterpart in the reference, which runs one curve per call
//! (src/secp256k1_ecdsa.rs:25-44).
use crate::ffi::*;
use crate::ShaderFailureError;

/// One item of a mixed batch.
pub enum Item<'a> {
    Secp256k1 { sig: &'a [u8; 64], msg: &'a [u8; 32] },
    Secp256r1 { sig: &'a [u8; 64], msg: &'a [u8; 32] },
    Ed25519 { sig: &'a [u8; 64], msg: &'a [u8; 32], key: &'a [u8; 32] },
}

/// Per item: `Ok(key)` (64 bytes) for a recovered ECDSA key, `Ok(vec![1])` /
/// `Ok(vec![0])` for an ed25519 verdict, `Err(status)` for an ECDSA signature
/// that does not recover.
pub fn verify_mixed(items: &[Item]) -> Result<Vec<Result<Vec<u8>, u8>>, ShaderFailureError> {
    let n = items.len();
    if n == 0 {
        return Ok(vec![]);
    }
    let mut curves = vec![0u8; n];
    let mut sigs = vec![0u8; 64 * n];
    let mut msgs = vec![0u8; 32 * n];
    let mut pks = vec![0u8; 32 * n];
    for (i, it) in items.iter().enumerate() {
        let (c, s, m) = match it {
            Item::Secp256k1 { sig, msg } => (SIGOPS_SECP256K1, *sig, *msg),
            Item::Secp256r1 { sig, msg } => (SIGOPS_SECP256R1, *sig, *msg),
            Item::Ed25519 { sig, msg, key } => {
                pks[32 * i..32 * i + 32].copy_from_slice(&key[..]);
                (SIGOPS_ED25519, *sig, *msg)
            }
        };
        curves[i] = c as u8;
        sigs[64 * i..64 * i + 64].copy_from_slice(&s[..]);
        msgs[32 * i..32 * i + 32].copy_from_slice(&m[..]);
    }
    let mut out = vec![0u8; 64 * n];
    let mut status = vec![0u8; n];
    let rc = unsafe {
        sigops_verify_mixed(std::ptr::null_mut(), curves.as_ptr(), sigs.as_ptr(), msgs.as_ptr(), pks.as_ptr(), n, out.as_mut_ptr(),
                            status.as_mut_ptr())
    };
    if rc != SIGOPS_OK {
        return Err(ShaderFailureError);
    }
    Ok((0..n)
        .map(|i| {
            if curves[i] == SIGOPS_ED25519 as u8 {
                Ok(vec![out[64 * i]])
            } else if status[i] == SIGOPS_ST_OK {
                Ok(out[64 * i..64 * i + 64].to_vec())
            } else {
                Err(status[i])
            }
        })
        .collect())
}
