"""Shared body of the secp256k1 / secp256r1 recovery modules."""

from __future__ import annotations

import numpy as np

from ._batch import as_rows, ptr, table_arg
from ._lib import SIGOPS_E_CUDA, SIGOPS_E_TIMEDOUT, SigopsError, lib
from .context import default_context


def _raise(code: int, where: str):
    from . import ShaderFailureError

    if code in (SIGOPS_E_CUDA, SIGOPS_E_TIMEDOUT):
        raise ShaderFailureError(str(SigopsError(code, where)))
    raise SigopsError(code, where)


def recover_arrays(fn_table, fn_single, signatures, messages, table_limbs, log_limb_size, ctx=None):
    """Returns (keys (n, 64) uint8, status (n,) uint8)."""
    sigs = as_rows(signatures, 64, "signatures")
    msgs = as_rows(messages, 32, "messages")
    if len(sigs) != len(msgs):
        raise ValueError(f"{len(sigs)} signatures but {len(msgs)} messages")
    n = len(sigs)
    out = np.zeros((n, 64), dtype=np.uint8)
    status = np.zeros(n, dtype=np.uint8)
    c = (ctx or default_context()).ptr
    if table_limbs is None:
        rc = getattr(lib, fn_single)(c, ptr(sigs), ptr(msgs), n, log_limb_size, ptr(out), ptr(status))
    else:
        t, tp, tn = table_arg(table_limbs)
        rc = getattr(lib, fn_table)(c, ptr(sigs), ptr(msgs), n, tp, tn, log_limb_size, ptr(out), ptr(status))
    if rc < 0:
        _raise(rc, fn_table if table_limbs is not None else fn_single)
    return out, status


def to_vecs(out: np.ndarray, status: np.ndarray) -> list[bytes]:
    """Per-item `Vec<u8>`: the 64 key bytes, or empty where recovery failed."""
    return [out[i].tobytes() if status[i] == 0 else b"" for i in range(len(status))]
