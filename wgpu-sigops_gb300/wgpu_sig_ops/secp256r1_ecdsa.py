"""secp256r1 ECDSA public-key recovery -- mirror of the reference module
`secp256r1_ecdsa` over libsigops.so.

Signatures are 64-byte fuel encodings (`fuel_types::Bytes64`: r || s big-endian, y parity
in bit 7 of byte 32), messages 32-byte digests (fuel `Message`).  Each
recovered key is 64 bytes (x || y big-endian); an item whose signature does not
recover (r or s out of range, r not on the curve, key at infinity) yields
`b""` -- the reference's CPU crates return `Err` for it -- and its status
code says why.
"""

from __future__ import annotations

from . import _ecdsa

_FN = "sigops_secp256r1_ecrecover"
_FN_SINGLE = "sigops_secp256r1_ecrecover_single_shader"


def ecrecover(signatures, messages, table_limbs, log_limb_size: int, ctx=None) -> list[bytes]:
    """`ecrecover(&Vec<Signature>, &Vec<Message>, &Vec<u32>, u32)` (src/secp256r1_ecdsa.rs (ecrecover)).

    `table_limbs` must equal `precompute.secp256r1_bases(log_limb_size)`."""
    out, status = _ecdsa.recover_arrays(_FN, _FN_SINGLE, signatures, messages, table_limbs, log_limb_size, ctx)
    return _ecdsa.to_vecs(out, status)


def ecrecover_single_shader(signatures, messages, log_limb_size: int, ctx=None) -> list[bytes]:
    """`ecrecover_single_shader` (src/secp256r1_ecdsa.rs (ecrecover_single_shader)): same result, no table argument."""
    out, status = _ecdsa.recover_arrays(_FN, _FN_SINGLE, signatures, messages, None, log_limb_size, ctx)
    return _ecdsa.to_vecs(out, status)


def ecrecover_arrays(signatures, messages, table_limbs=None, log_limb_size: int = 13, ctx=None):
    """Array form: returns (keys (n, 64) uint8, status (n,) uint8)."""
    return _ecdsa.recover_arrays(_FN, _FN_SINGLE, signatures, messages, table_limbs, log_limb_size, ctx)
