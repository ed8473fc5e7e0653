"""The C-ABI library: loads, exports every symbol include/sigops.h declares,
and its CPU-only entry points (tables) work without a GPU."""
import ctypes
import os
import re

import pytest

from oracle import sigops_oracle as o
from tests._paths import ROOT, build_lib


@pytest.fixture(scope="module")
def lib():
    return ctypes.CDLL(build_lib())


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "sigops.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sigops_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name


def test_python_binding_covers_header():
    import wgpu_sig_ops._lib as L

    assert set(declared_symbols()) == set(L.SIGNATURES)


@pytest.mark.parametrize("curve,fn", [(0, o.secp256k1_bases), (1, o.secp256r1_bases), (2, o.ed25519_bases)])
def test_bases_match_oracle(curve, fn):
    from wgpu_sig_ops import precompute

    mod = [precompute.secp256k1_bases, precompute.secp256r1_bases, precompute.ed25519_bases][curve]
    for L in (11, 13, 15):
        assert mod(L) == fn(L)


def test_check_table(lib):
    import numpy as np

    from wgpu_sig_ops import _lib as L
    from wgpu_sig_ops import precompute

    t = np.array(precompute.secp256k1_bases(13), dtype=np.uint32)
    p = t.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    assert L.lib.sigops_check_table(0, p, t.size, 13) == 0
    assert L.lib.sigops_check_table(1, p, t.size, 13) == L.SIGOPS_E_TABLE
    assert L.lib.sigops_check_table(0, p, t.size - 1, 13) == L.SIGOPS_E_TABLE
    t[5] ^= 1
    assert L.lib.sigops_check_table(0, p, t.size, 13) == L.SIGOPS_E_TABLE
    assert L.lib.sigops_bases_len(0, 16) == L.SIGOPS_E_INVAL
    assert L.lib.sigops_bases_len(3, 13) == L.SIGOPS_E_INVAL
    assert L.lib.sigops_bases_len(2, 13) == 16 * 3 * 20


def test_no_device_is_reported(lib):
    """Without a GPU, creating a context fails cleanly (no CPU fallback)."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from wgpu_sig_ops import _lib as L

    assert not L.lib.sigops_create(0)
    assert b"device" in L.lib.sigops_last_error()


def test_mixed_batch_size_limit(lib):
    """The mixed engine's index lists hold 32-bit item indices: larger batches
    are refused before any device work (no GPU needed)."""
    from wgpu_sig_ops import _lib as L

    buf = ctypes.create_string_buffer(64)
    n = 2**32
    assert L.lib.sigops_verify_mixed(None, buf, buf, buf, buf, n, buf, buf) == L.SIGOPS_E_RANGE
    assert b"32-bit" in L.lib.sigops_last_error()
    assert L.lib.sigops_verify_mixed_device(None, buf, buf, buf, buf, n, buf, buf, None) == L.SIGOPS_E_RANGE


def test_rust_binding_covers_header():
    """The Rust crate's raw declarations (wgpu-sigops_gb300/rust/src/ffi.rs,
    not compiled here: no Rust toolchain) name every function the header
    declares, and no other."""
    src = open(os.path.join(ROOT, "wgpu-sigops_gb300", "rust", "src", "ffi.rs")).read()
    rust = set(re.findall(r"\bpub fn (sigops_[a-z0-9_]+)\s*\(", src))
    assert rust == set(declared_symbols())
