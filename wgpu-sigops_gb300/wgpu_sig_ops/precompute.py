"""Generator tables -- mirror of the reference module `precompute`
(src/precompute.rs:12-69), computed by libsigops.so on the CPU (no GPU needed)."""

from __future__ import annotations

import ctypes

import numpy as np

from ._lib import ED25519, SECP256K1, SECP256R1, check, lib

WINDOW_SIZE = 4  # src/precompute.rs:12


def _bases(curve: int, log_limb_size: int) -> list[int]:
    n = check(lib.sigops_bases_len(curve, log_limb_size), "sigops_bases_len")
    buf = np.zeros(n, dtype=np.uint32)
    check(lib.sigops_bases(curve, log_limb_size, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), n), "sigops_bases")
    return [int(v) for v in buf]


def secp256k1_bases(log_limb_size: int) -> list[int]:
    return _bases(SECP256K1, log_limb_size)


def secp256r1_bases(log_limb_size: int) -> list[int]:
    return _bases(SECP256R1, log_limb_size)


def ed25519_bases(log_limb_size: int) -> list[int]:
    return _bases(ED25519, log_limb_size)
