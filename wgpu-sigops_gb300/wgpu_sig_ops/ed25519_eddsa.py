"""ed25519 verification -- mirror of the reference module `ed25519_eddsa`
over libsigops.so, with ed25519-dalek 2.1.1 `VerifyingKey::verify` semantics
(non-canonical S >= l rejected; the R bytes compared as given).

Signatures are 64 bytes (R || S, `ed25519_dalek::Signature::to_bytes()`),
messages 32 bytes (fuel `Message`), keys 32 bytes (`VerifyingKey::to_bytes()`).
"""

from __future__ import annotations

import numpy as np

from ._batch import as_rows, ptr, table_arg
from ._ecdsa import _raise
from ._lib import lib
from .context import default_context


def ecverify_arrays(signatures, messages, verifying_keys, table_limbs=None, log_limb_size: int = 13, ctx=None):
    """Array form: returns (valid (n,) uint8 0/1, status (n,) uint8)."""
    sigs = as_rows(signatures, 64, "signatures")
    msgs = as_rows(messages, 32, "messages")
    pks = as_rows(verifying_keys, 32, "verifying_keys")
    if not (len(sigs) == len(msgs) == len(pks)):
        raise ValueError(f"lengths differ: {len(sigs)} signatures, {len(msgs)} messages, {len(pks)} keys")
    n = len(sigs)
    valid = np.zeros(n, dtype=np.uint8)
    status = np.zeros(n, dtype=np.uint8)
    c = (ctx or default_context()).ptr
    if table_limbs is None:
        rc = lib.sigops_ed25519_ecverify_single(c, ptr(sigs), ptr(msgs), ptr(pks), n, log_limb_size, ptr(valid), ptr(status))
        where = "sigops_ed25519_ecverify_single"
    else:
        t, tp, tn = table_arg(table_limbs)
        rc = lib.sigops_ed25519_ecverify(c, ptr(sigs), ptr(msgs), ptr(pks), n, tp, tn, log_limb_size, ptr(valid), ptr(status))
        where = "sigops_ed25519_ecverify"
    if rc < 0:
        _raise(rc, where)
    return valid, status


def ecverify(signatures, messages, verifying_keys, table_limbs, log_limb_size: int, ctx=None) -> list[bool]:
    """`ecverify(&Vec<Signature>, &Vec<Message>, &Vec<VerifyingKey>, &Vec<u32>, u32)`
    (src/ed25519_eddsa.rs:67-257)."""
    valid, _ = ecverify_arrays(signatures, messages, verifying_keys, table_limbs, log_limb_size, ctx)
    return [bool(v) for v in valid]


def ecverify_single(signatures, messages, verifying_keys, log_limb_size: int, ctx=None) -> list[bool]:
    """`ecverify_single` (src/ed25519_eddsa.rs:259-324)."""
    valid, _ = ecverify_arrays(signatures, messages, verifying_keys, None, log_limb_size, ctx)
    return [bool(v) for v in valid]


def verify_raw_arrays(signatures, messages, verifying_keys, ctx=None):
    """Messages of any length (list of bytes-like): returns (valid (n,) uint8
    0/1, status (n,) uint8).  No counterpart in the reference, whose API takes
    32-byte messages only."""
    sigs = as_rows(signatures, 64, "signatures")
    pks = as_rows(verifying_keys, 32, "verifying_keys")
    msgs = [bytes(m) for m in messages]
    if not (len(sigs) == len(msgs) == len(pks)):
        raise ValueError(f"lengths differ: {len(sigs)} signatures, {len(msgs)} messages, {len(pks)} keys")
    n = len(sigs)
    lens = np.array([len(m) for m in msgs], dtype=np.uint32)
    offsets = np.zeros(n, dtype=np.uint64)
    if n:
        offsets[1:] = np.cumsum(lens[:-1], dtype=np.uint64)
    blob = np.frombuffer(b"".join(msgs), dtype=np.uint8) if n else np.zeros(0, np.uint8)
    blob = np.ascontiguousarray(blob) if len(blob) else np.zeros(1, np.uint8)
    valid = np.zeros(n, dtype=np.uint8)
    status = np.zeros(n, dtype=np.uint8)
    c = (ctx or default_context()).ptr
    rc = lib.sigops_ed25519_verify_raw(c, ptr(sigs), ptr(blob), int(lens.sum()), ptr(offsets), ptr(lens), ptr(pks), n, ptr(valid),
                                       ptr(status))
    if rc < 0:
        _raise(rc, "sigops_ed25519_verify_raw")
    return valid, status


def verify_raw(signatures, messages, verifying_keys, ctx=None) -> list[bool]:
    """ed25519-dalek `VerifyingKey::verify(&[u8], &Signature)` per item, for
    messages of any length."""
    valid, _ = verify_raw_arrays(signatures, messages, verifying_keys, ctx)
    return [bool(v) for v in valid]
