//! precompute::{secp256k1,secp256r1,ed25519}_bases (src/precompute.rs:36-69):
//! the table of [1..16]G in Montgomery form with `log_limb_size`-bit limbs,
//! bit-identical to the reference.  CPU only.
use crate::ffi::*;

pub fn secp256k1_bases(log_limb_size: u32) -> Vec<u32> {
    bases(SIGOPS_SECP256K1, log_limb_size)
}

pub fn secp256r1_bases(log_limb_size: u32) -> Vec<u32> {
    bases(SIGOPS_SECP256R1, log_limb_size)
}

pub fn ed25519_bases(log_limb_size: u32) -> Vec<u32> {
    bases(SIGOPS_ED25519, log_limb_size)
}

fn bases(curve: i32, log_limb_size: u32) -> Vec<u32> {
    let n = unsafe { sigops_bases_len(curve, log_limb_size) };
    assert!(n > 0, "log_limb_size must be in 11..=15");
    let mut v = vec![0u32; n as usize];
    let got = unsafe { sigops_bases(curve, log_limb_size, v.as_mut_ptr(), v.len()) };
    assert_eq!(got, n);
    v
}
