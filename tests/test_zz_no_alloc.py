"""The allocation-free entry point (sigops_verify_mixed_noalloc).

It serves callers that cannot allocate device memory per call -- processes
whose GPU memory belongs to another allocator or to a budget reserved at
start-up, and latency-critical threads that cannot absorb cudaMalloc's implicit
synchronisation.  Called through the C ABI, two calls in a row, its results
must equal those of the context-based entry point on the same inputs, bit for
bit; so must a call at the size limit, whose index lists fill the static
scratch exactly.  Its device error word reads back clear.  A fresh process
whose very first CUDA work is this call, on a non-blocking stream, must match
the oracle.  This file is collected last on purpose, and also passes alone in a
fresh process."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _device_batch(W, torch):
    dev = torch.device("cuda")
    return {
        "cur": torch.from_numpy(W.curves).to(dev),
        "sig": torch.from_numpy(W.sigs).to(dev),
        "msg": torch.from_numpy(W.msgs).to(dev),
        "pk": torch.from_numpy(W.pks).to(dev),
    }


def _compare_with_context(W, torch, stream):
    import wgpu_sig_ops as w
    from wgpu_sig_ops import workload as wl
    from wgpu_sig_ops._lib import check, lib

    ctx = w.default_context()
    d = _device_batch(W, torch)
    n = W.n
    ref_out = torch.zeros((n, 64), dtype=torch.uint8, device="cuda")
    ref_st = torch.zeros(n, dtype=torch.uint8, device="cuda")
    got_out = torch.zeros((n, 64), dtype=torch.uint8, device="cuda")
    got_st = torch.full((n,), 0xFF, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    check(lib.sigops_verify_mixed_device(ctx.ptr, d["cur"].data_ptr(), d["sig"].data_ptr(), d["msg"].data_ptr(), d["pk"].data_ptr(),
                                         n, ref_out.data_ptr(), ref_st.data_ptr(), None), "reference entry point")
    check(lib.sigops_sync(ctx.ptr), "sync")
    with torch.cuda.stream(stream):
        rc = lib.sigops_verify_mixed_noalloc(d["cur"].data_ptr(), d["sig"].data_ptr(), d["msg"].data_ptr(), d["pk"].data_ptr(), n,
                                             got_out.data_ptr(), got_st.data_ptr(), stream.cuda_stream)
    assert rc == 0
    assert lib.sigops_noalloc_status(stream.cuda_stream) == 0  # waits for the call; no device-side error
    assert (got_st.cpu().numpy() != 0xFF).all()
    assert torch.equal(got_out, ref_out) and torch.equal(got_st, ref_st)
    chk = wl.expected_check(W, got_out.cpu().numpy(), got_st.cpu().numpy())
    assert chk["mismatches"] == 0, chk


def test_noalloc_matches_context_entry_point_twice():
    torch = pytest.importorskip("torch")
    from wgpu_sig_ops import workload as wl

    # two different batches, so the second call cannot pass on stale scratch
    stream = torch.cuda.Stream()
    for W in (wl.config("c4", n=6000, seed=91), wl.config("c4", n=4500, seed=92)):
        _compare_with_context(W, torch, stream)


def test_noalloc_at_the_size_limit():
    torch = pytest.importorskip("torch")
    from wgpu_sig_ops import workload as wl
    from wgpu_sig_ops._lib import lib  # noqa: F401

    # 65,536 items: the three index lists fill the static scratch exactly
    W = wl.config("c4", n=65536, seed=93)
    assert W.n == 65536
    _compare_with_context(W, torch, torch.cuda.Stream())


def test_noalloc_host_side_checks():
    pytest.importorskip("torch")
    import wgpu_sig_ops  # noqa: F401  (loads the library)
    from wgpu_sig_ops._lib import SIGOPS_E_INVAL, SIGOPS_E_RANGE, lib

    aligned = ctypes.c_void_p(256)
    # refused on the host before anything is launched
    assert lib.sigops_verify_mixed_noalloc(aligned, aligned, aligned, aligned, 65536 + 1, aligned, aligned, None) == SIGOPS_E_RANGE
    assert lib.sigops_verify_mixed_noalloc(aligned, aligned, aligned, aligned, 0, aligned, aligned, None) == 0
    odd = ctypes.c_void_p(256 + 4)
    assert lib.sigops_verify_mixed_noalloc(aligned, odd, aligned, aligned, 16, aligned, aligned, None) == SIGOPS_E_INVAL
    assert lib.sigops_verify_mixed_noalloc(aligned, aligned, aligned, aligned, 16, odd, aligned, None) == SIGOPS_E_INVAL
    assert lib.sigops_verify_mixed_noalloc(None, aligned, aligned, aligned, 16, aligned, aligned, None) == SIGOPS_E_INVAL


_FRESH = r"""
import sys
sys.path[:0] = [{root!r}, {pkg!r}]
import numpy as np, torch
from oracle import c_oracle
rng = np.random.Generator(np.random.PCG64(94))
n = 300
curves = rng.integers(0, 3, size=n, dtype=np.uint8)
sigs = np.zeros((n, 64), np.uint8); msgs = rng.integers(0, 256, size=(n, 32), dtype=np.uint8); pks = np.zeros((n, 32), np.uint8)
N = {{0: 0xFFFFFFFFFFFFFFFFFFFFFFFFFFFFFFFEBAAEDCE6AF48A03BBFD25E8CD0364141, 1: 0xFFFFFFFF00000000FFFFFFFFFFFFFFFFBCE6FAADA7179E84F3B9CAC2FC632551}}
for i in range(n):
    c = int(curves[i])
    if c == 2:
        s, pk = c_oracle.ed25519_sign(rng.bytes(32), msgs[i].tobytes())
        sigs[i] = np.frombuffer(s, np.uint8); pks[i] = np.frombuffer(pk, np.uint8)
    else:
        while True:
            d = int.from_bytes(rng.bytes(32), "big") % N[c] or 1
            k = int.from_bytes(rng.bytes(32), "big") % N[c] or 1
            r = c_oracle.ecdsa_sign(c, d, msgs[i].tobytes(), k)
            if r:
                sigs[i] = np.frombuffer(r[0], np.uint8); break
sigs[7, 40] ^= 1  # one tampered item
want_out, want_st = c_oracle.batch_mixed(curves, sigs, msgs, pks)
from wgpu_sig_ops._lib import lib  # no context is created: the next call is the first CUDA work of the library
stream = torch.cuda.Stream()  # non-blocking
with torch.cuda.stream(stream):
    t = [torch.from_numpy(a).cuda() for a in (curves, sigs, msgs, pks)]
    out = torch.zeros((n, 64), dtype=torch.uint8, device="cuda"); st = torch.full((n,), 0xFF, dtype=torch.uint8, device="cuda")
stream.synchronize()
rc = lib.sigops_verify_mixed_noalloc(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(), n, out.data_ptr(), st.data_ptr(),
                                     stream.cuda_stream)
assert rc == 0, rc
assert lib.sigops_noalloc_status(stream.cuda_stream) == 0
assert (st.cpu().numpy() == want_st).all() and (out.cpu().numpy() == want_out).all()
print("fresh ok")
"""


def test_noalloc_first_call_of_a_fresh_process_on_a_nonblocking_stream():
    pytest.importorskip("torch")
    code = _FRESH.format(root=ROOT, pkg=os.path.join(ROOT, "wgpu-sigops_gb300"))
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0 and "fresh ok" in p.stdout, p.stdout + p.stderr
