"""The allocation-free entry point (sigops_verify_mixed_noalloc).

It serves callers that cannot allocate device memory per call -- processes
whose GPU memory belongs to another allocator or to a budget reserved at
start-up, and latency-critical threads that cannot absorb cudaMalloc's implicit
synchronisation.  Called through the C ABI, two calls in a row, its results
must equal those of the context-based entry point on the same inputs, bit for
bit.  This file is collected last on purpose, and also passes alone in a fresh
process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_batch(W, torch):
    dev = torch.device("cuda")
    return {
        "cur": torch.from_numpy(W.curves).to(dev),
        "sig": torch.from_numpy(W.sigs).to(dev),
        "msg": torch.from_numpy(W.msgs).to(dev),
        "pk": torch.from_numpy(W.pks).to(dev),
    }


def test_noalloc_matches_context_entry_point_twice():
    torch = pytest.importorskip("torch")
    import wgpu_sig_ops as w
    from wgpu_sig_ops import workload as wl
    from wgpu_sig_ops._lib import check, lib

    ctx = w.default_context()
    # two different batches, so the second call cannot pass on stale scratch
    batches = [wl.config("c4", n=6000, seed=91), wl.config("c4", n=4500, seed=92)]
    stream = torch.cuda.Stream()
    for W in batches:
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
        stream.synchronize()
        assert (got_st.cpu().numpy() != 0xFF).all()
        assert torch.equal(got_out, ref_out) and torch.equal(got_st, ref_st)
        chk = wl.expected_check(W, got_out.cpu().numpy(), got_st.cpu().numpy())
        assert chk["mismatches"] == 0, chk


def test_noalloc_rejects_oversize_batch():
    pytest.importorskip("torch")
    import wgpu_sig_ops  # noqa: F401  (loads the library)
    from wgpu_sig_ops._lib import SIGOPS_E_RANGE, lib

    n = 65536 + 1
    dummy = ctypes.c_void_p(16)
    assert lib.sigops_verify_mixed_noalloc(dummy, dummy, dummy, dummy, n, dummy, dummy, None) == SIGOPS_E_RANGE
