"""Threads per signature: secp256k1 recovery by a lane pair per signature (the
GLV halves of both scalars on the two lanes) gives the same keys and statuses
as one thread per signature, for valid, tampered and no-point items and for a
count that leaves a lane pair without an item."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_lane_pair_equals_one_lane():
    torch = pytest.importorskip("torch")
    import ctypes

    import wgpu_sig_ops as w
    from wgpu_sig_ops import workload as wl
    from wgpu_sig_ops._lib import check, lib

    W = wl.config("c4", n=20000, seed=61)
    sel = np.nonzero(W.curves == 0)[0][:4999]  # odd count: the last pair's partner has no item
    sigs = np.ascontiguousarray(W.sigs[sel])
    msgs = np.ascontiguousarray(W.msgs[sel])
    n = len(sel)
    d_sig = torch.from_numpy(sigs).cuda()
    d_msg = torch.from_numpy(msgs).cuda()
    res = {}
    for lanes in (1, 2):
        out = torch.zeros((n, 64), dtype=torch.uint8, device="cuda")
        st = torch.full((n,), 0xFF, dtype=torch.uint8, device="cuda")
        ms = ctypes.c_float()
        torch.cuda.synchronize()
        check(lib.sigops_probe_k1_lanes(w.default_context().ptr, lanes, 0, d_sig.data_ptr(), d_msg.data_ptr(), n, out.data_ptr(),
                                        st.data_ptr(), ctypes.byref(ms)), "sigops_probe_k1_lanes")
        res[lanes] = (out.cpu().numpy(), st.cpu().numpy())
    assert (res[1][1] != 0xFF).all()
    assert (res[1][0] == res[2][0]).all() and (res[1][1] == res[2][1]).all()
    # and both equal the plain kernel's
    ref_out, ref_st = w.batch.verify_mixed(np.zeros(n, np.uint8), sigs, msgs, np.zeros((n, 32), np.uint8))
    assert (res[1][0] == ref_out).all() and (res[1][1] == ref_st).all()
    assert (ref_st != 0).any() and (ref_st == 0).any()  # the sample holds failing items too


def test_phase_probe_equals_plain():
    """Persistent warps, free-running or block-synchronised, recover the same
    keys and statuses as the plain kernel, with an item count that leaves the
    last group partial and a synchronised block's last round partly empty, and
    time every group."""
    torch = pytest.importorskip("torch")
    import ctypes

    import wgpu_sig_ops as w
    from wgpu_sig_ops import workload as wl
    from wgpu_sig_ops._lib import check, lib

    W = wl.config("c4", n=20000, seed=62)
    sel = np.nonzero(W.curves == 0)[0][:5001]
    sigs = np.ascontiguousarray(W.sigs[sel])
    msgs = np.ascontiguousarray(W.msgs[sel])
    n = len(sel)
    groups = (n + 31) // 32
    d_sig = torch.from_numpy(sigs).cuda()
    d_msg = torch.from_numpy(msgs).cuda()
    ref_out, ref_st = w.batch.verify_mixed(np.zeros(n, np.uint8), sigs, msgs, np.zeros((n, 32), np.uint8))
    assert (ref_st != 0).any() and (ref_st == 0).any()
    for sync in (0, 1):
        out = torch.zeros((n, 64), dtype=torch.uint8, device="cuda")
        st = torch.full((n,), 0xFF, dtype=torch.uint8, device="cuda")
        times = torch.zeros(2 * groups, dtype=torch.int64, device="cuda")
        ms = ctypes.c_float()
        torch.cuda.synchronize()
        check(lib.sigops_probe_phase(w.default_context().ptr, sync, d_sig.data_ptr(), d_msg.data_ptr(), n, out.data_ptr(), st.data_ptr(),
                                     times.data_ptr(), ctypes.byref(ms)), "sigops_probe_phase")
        assert (out.cpu().numpy() == ref_out).all() and (st.cpu().numpy() == ref_st).all(), sync
        t = times.cpu().numpy().reshape(-1, 2)
        assert (t[:, 0] > 0).all() and (t[:, 1] >= t[:, 0]).all(), sync
        assert ms.value > 0
