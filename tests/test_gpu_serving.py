"""The continuous-batching serving loop: each request's result is the same
alone and in the mix, requests that arrive while others run join later
launches, and admission limits hold."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def w():
    import wgpu_sig_ops

    return wgpu_sig_ops


@pytest.fixture(scope="module")
def W(w):
    from wgpu_sig_ops import workload as wl

    return wl.config("c4", n=40000, seed=77)


@pytest.mark.parametrize("variant", [0, 40], ids=["fused", "single-curve"])
def test_alone_equals_in_the_mix(w, W, variant):
    from wgpu_sig_ops.serving import Server, curve_sorted_pool, request_stream

    ctx = w.default_context()
    pool, regions = curve_sorted_pool(W)
    offs, cnts, arr = request_stream(regions, 0.0, 0.0, seed=3, n_requests=120)
    # reference: every request alone, one at a time, through its own server call
    srv = Server(ctx, slots=3, slot_items=8192, variant=variant)
    alone = []
    for o, c in zip(offs, cnts):
        sl = slice(int(o), int(o) + int(c))
        h = srv.submit(pool["curves"][sl], pool["sigs"][sl], pool["msgs"][sl], pool["pks"][sl])
        out, st, _ = srv.wait(h)
        alone.append((out, st))
    # the same requests submitted together (packed into shared launches)
    handles = []
    for o, c in zip(offs, cnts):
        sl = slice(int(o), int(o) + int(c))
        handles.append(srv.submit(pool["curves"][sl], pool["sigs"][sl], pool["msgs"][sl], pool["pks"][sl]))
    before = srv.stats()["launches"]
    mixed = [srv.wait(h) for h in handles]
    srv.close()
    for (a_out, a_st), (m_out, m_st, _) in zip(alone, mixed):
        assert (a_out == m_out).all() and (a_st == m_st).all()
    # and both equal the batched engine on the whole pool
    ref_out, ref_st = w.batch.verify_mixed(pool["curves"], pool["sigs"], pool["msgs"], pool["pks"])
    for (o, c), (m_out, m_st, _) in zip(zip(offs, cnts), mixed):
        assert (m_out == ref_out[int(o):int(o) + int(c)]).all() and (m_st == ref_st[int(o):int(o) + int(c)]).all()


def test_continuous_batching_packs_arrivals(w, W):
    """120 requests submitted back to back while the first launch runs are
    packed into far fewer launches than requests."""
    from wgpu_sig_ops.serving import Server, curve_sorted_pool, request_stream

    ctx = w.default_context()
    pool, regions = curve_sorted_pool(W)
    offs, cnts, arr = request_stream(regions, 0.0, 0.0, seed=4, n_requests=120)
    srv = Server(ctx, slots=2, slot_items=32768)
    rc, lat, wall, out, st = srv.run_load(pool, offs, cnts, arr)
    s = srv.stats()
    srv.close()
    assert rc == 0 and (lat > 0).all()
    assert s["requests_done"] == 120 and s["launches"] < 60
    ref_out, ref_st = w.batch.verify_mixed(pool["curves"], pool["sigs"], pool["msgs"], pool["pks"])
    for o, c in zip(offs, cnts):
        sl = slice(int(o), int(o) + int(c))
        assert (out[sl] == ref_out[sl]).all() and (st[sl] == ref_st[sl]).all()


def test_admission_limits(w, W):
    from wgpu_sig_ops._lib import SIGOPS_E_RANGE, SigopsError
    from wgpu_sig_ops.serving import Server

    srv = Server(w.default_context(), slots=1, slot_items=1024)
    with pytest.raises(SigopsError) as e:
        srv.submit(W.curves[:2000], W.sigs[:2000], W.msgs[:2000], W.pks[:2000])
    assert e.value.code == SIGOPS_E_RANGE
    h = srv.submit(0, W.sigs[:1], W.msgs[:1])
    out, st, lat = srv.wait(h)
    assert lat > 0
    srv.close()


def test_poisson_load_short(w, W):
    from wgpu_sig_ops.serving import measure

    res = measure(w.default_context(), W, loads=(0.5,), seconds=2.0, sat_items=200000, slot_items=16384)
    lvl = res["levels"][0]
    assert res["saturation_sigs_per_s"] > 0 and lvl["refused"] == 0 and lvl["p50_ms"] > 0
