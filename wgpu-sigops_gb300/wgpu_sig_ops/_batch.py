"""Packing helpers shared by the per-curve modules."""

from __future__ import annotations

import numpy as np


def as_rows(items, width: int, what: str) -> np.ndarray:
    """Sequence of ``width``-byte objects (bytes, bytearray, numpy rows) or an
    (n, width) uint8 array -> C-contiguous (n, width) uint8 array."""
    if isinstance(items, np.ndarray):
        a = np.ascontiguousarray(items, dtype=np.uint8)
        if a.ndim == 1 and a.size % width == 0:
            a = a.reshape(-1, width)
        if a.ndim != 2 or a.shape[1] != width:
            raise ValueError(f"{what}: expected shape (n, {width}), got {a.shape}")
        return a
    rows = [bytes(x) for x in items]
    for r in rows:
        if len(r) != width:
            raise ValueError(f"{what}: every item must be {width} bytes, got {len(r)}")
    if not rows:
        return np.zeros((0, width), dtype=np.uint8)
    return np.frombuffer(b"".join(rows), dtype=np.uint8).reshape(-1, width).copy()


def ptr(a: np.ndarray):
    return a.ctypes.data if a.size else None


def table_arg(table_limbs):
    import ctypes

    t = np.ascontiguousarray(np.asarray(table_limbs, dtype=np.uint32))
    return t, t.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), t.size
