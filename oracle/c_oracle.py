"""ctypes binding of the oracle's C restatement (oracle/csrc/sigops_oracle.c).
Test infrastructure only: the checker for large batches and the CPU baseline."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_oracle.build())
        _vp, _sz = ctypes.c_void_p, ctypes.c_size_t
        _lib.sigops_oracle_batch.argtypes = [ctypes.c_int, _vp, _vp, _vp, _sz, _vp, _vp, ctypes.c_int]
        _lib.sigops_oracle_batch_mixed.argtypes = [_vp, _vp, _vp, _vp, _sz, _vp, _vp, ctypes.c_int]
        _lib.sigops_oracle_ecdsa_sign.argtypes = [ctypes.c_int, _vp, _vp, _vp, _vp, _vp]
        _lib.sigops_oracle_ed25519_sign.argtypes = [_vp, _vp, _vp, _vp]
        _lib.sigops_oracle_secp256k1_recover.argtypes = [_vp, _vp, _vp]
        _lib.sigops_oracle_secp256r1_recover.argtypes = [_vp, _vp, _vp]
        _lib.sigops_oracle_ed25519_verify.argtypes = [_vp, _vp, _vp]
    return _lib


def _p(a):
    return a.ctypes.data if a is not None and a.size else None


def batch(curve: int, sigs: np.ndarray, msgs: np.ndarray, pks: np.ndarray | None = None, threads: int | None = None):
    """Returns (out, status): out (n, 64) keys for ECDSA or (n,) validity for ed25519."""
    sigs = np.ascontiguousarray(sigs, dtype=np.uint8).reshape(-1, 64)
    msgs = np.ascontiguousarray(msgs, dtype=np.uint8).reshape(-1, 32)
    n = len(sigs)
    if pks is not None:
        pks = np.ascontiguousarray(pks, dtype=np.uint8).reshape(-1, 32)
    out = np.zeros((n, 64) if curve != 2 else n, dtype=np.uint8)
    status = np.zeros(n, dtype=np.uint8)
    lib().sigops_oracle_batch(curve, _p(sigs), _p(msgs), _p(pks), n, _p(out), _p(status), threads or os.cpu_count() or 1)
    return out, status


def batch_mixed(curves, sigs, msgs, pks, threads: int | None = None):
    curves = np.ascontiguousarray(curves, dtype=np.uint8)
    sigs = np.ascontiguousarray(sigs, dtype=np.uint8).reshape(-1, 64)
    msgs = np.ascontiguousarray(msgs, dtype=np.uint8).reshape(-1, 32)
    pks = np.ascontiguousarray(pks, dtype=np.uint8).reshape(-1, 32)
    n = len(curves)
    out = np.zeros((n, 64), dtype=np.uint8)
    status = np.zeros(n, dtype=np.uint8)
    lib().sigops_oracle_batch_mixed(_p(curves), _p(sigs), _p(msgs), _p(pks), n, _p(out), _p(status), threads or os.cpu_count() or 1)
    return out, status


def ecdsa_sign(curve: int, d: int, msg: bytes, k: int) -> tuple[bytes, bytes] | None:
    sig = ctypes.create_string_buffer(64)
    pub = ctypes.create_string_buffer(64)
    rc = lib().sigops_oracle_ecdsa_sign(curve, d.to_bytes(32, "big"), msg, k.to_bytes(32, "big"), sig, pub)
    return None if rc else (sig.raw, pub.raw)


def ed25519_sign(seed: bytes, msg: bytes) -> tuple[bytes, bytes]:
    sig = ctypes.create_string_buffer(64)
    pk = ctypes.create_string_buffer(32)
    lib().sigops_oracle_ed25519_sign(seed, msg, sig, pk)
    return sig.raw, pk.raw
