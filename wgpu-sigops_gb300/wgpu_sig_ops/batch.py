"""Batched mixed-curve verification: one call of the batched engine per batch
(a classify kernel, then the context's launch variant)."""

from __future__ import annotations

import ctypes

import numpy as np

from ._batch import as_rows, ptr
from ._ecdsa import _raise
from ._lib import check, lib
from .context import default_context


def verify_mixed(curves, signatures, messages, verifying_keys, ctx=None):
    """Returns (out (n, 64) uint8, status (n,) uint8).  ECDSA items: recovered
    key (zero when status != OK); ed25519 items: out[i, 0] = valid."""
    cur = np.ascontiguousarray(np.asarray(curves, dtype=np.uint8))
    sigs = as_rows(signatures, 64, "signatures")
    msgs = as_rows(messages, 32, "messages")
    pks = as_rows(verifying_keys, 32, "verifying_keys")
    n = len(cur)
    if not (len(sigs) == len(msgs) == len(pks) == n):
        raise ValueError("curves, signatures, messages and keys must have the same length")
    out = np.zeros((n, 64), dtype=np.uint8)
    status = np.zeros(n, dtype=np.uint8)
    rc = lib.sigops_verify_mixed((ctx or default_context()).ptr, ptr(cur), ptr(sigs), ptr(msgs), ptr(pks), n, ptr(out), ptr(status))
    if rc < 0:
        _raise(rc, "sigops_verify_mixed")
    return out, status


def verify_mixed_into(ctx, curves: np.ndarray, sigs: np.ndarray, msgs: np.ndarray, pks: np.ndarray, out: np.ndarray, status: np.ndarray):
    """Zero-copy form over caller-owned (ideally page-locked) host arrays."""
    n = len(curves)
    rc = lib.sigops_verify_mixed(ctx.ptr, ptr(curves), ptr(sigs), ptr(msgs), ptr(pks), n, ptr(out), ptr(status))
    if rc < 0:
        _raise(rc, "sigops_verify_mixed")


class MixedPlan:
    """A CUDA graph of one batched step over fixed device buffers."""

    def __init__(self, ctx, d_curves: int, d_sigs: int, d_msgs: int, d_pks: int, n: int, d_out: int, d_status: int):
        self.ctx = ctx
        p = ctypes.c_void_p()
        check(lib.sigops_mixed_plan_create(ctx.ptr, d_curves, d_sigs, d_msgs, d_pks, n, d_out, d_status, ctypes.byref(p)),
              "sigops_mixed_plan_create")
        self.ptr = p.value

    def launch(self, stream: int | None = None):
        check(lib.sigops_mixed_plan_launch(self.ptr, stream or None), "sigops_mixed_plan_launch")

    def close(self):
        if self.ptr:
            lib.sigops_mixed_plan_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
