"""The continuous-batching serving loop: each request's result is the same
alone and in the mix, for every shape of the persistent kernel; requests that
arrive while others run are worked off by the running kernel (no launch per
request); admission refuses what does not fit; the adaptive shape follows the
load; cancel, the kernel's idle close and relaunch, a dispatcher that stops and
failed allocations are handled without a device fault."""
import time

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


@pytest.fixture(scope="module")
def ref(w, W):
    from wgpu_sig_ops.serving import curve_sorted_pool

    pool, regions = curve_sorted_pool(W)
    out, st = w.batch.verify_mixed(pool["curves"], pool["sigs"], pool["msgs"], pool["pks"])
    return pool, regions, out, st


@pytest.mark.parametrize("shape", [0, 1, 2], ids=["256x1", "128x3", "256x2"])
def test_alone_equals_in_the_mix(w, ref, shape):
    from wgpu_sig_ops.serving import Server, request_stream

    pool, regions, ref_out, ref_st = ref
    offs, cnts, arr = request_stream(regions, 0.0, 0.0, seed=3, n_requests=120)
    srv = Server(w.default_context(), slots=16, slot_items=8192, variant=shape)
    # every request alone, one at a time
    alone = []
    for o, c in zip(offs, cnts):
        sl = slice(int(o), int(o) + int(c))
        h = srv.submit(pool["curves"][sl], pool["sigs"][sl], pool["msgs"][sl], pool["pks"][sl])
        out, st, _ = srv.wait(h)
        alone.append((out, st))
    # the same requests submitted back to back, worked off together
    handles = []
    for o, c in zip(offs, cnts):
        sl = slice(int(o), int(o) + int(c))
        handles.append(srv.submit(pool["curves"][sl], pool["sigs"][sl], pool["msgs"][sl], pool["pks"][sl]))
    mixed = [srv.wait(h) for h in handles]
    srv.close()
    for (a_out, a_st), (m_out, m_st, _) in zip(alone, mixed):
        assert (a_out == m_out).all() and (a_st == m_st).all()
    # and both equal the batched engine on the whole pool
    for (o, c), (m_out, m_st, _) in zip(zip(offs, cnts), mixed):
        assert (m_out == ref_out[int(o):int(o) + int(c)]).all() and (m_st == ref_st[int(o):int(o) + int(c)]).all()


def test_mixed_curve_requests(w, W):
    """Requests whose items mix the three curves are regrouped by curve on
    submit; results come back in the caller's order."""
    from wgpu_sig_ops.serving import Server

    srv = Server(w.default_context(), slots=8, slot_items=4096)
    ref_out, ref_st = w.batch.verify_mixed(W.curves[:12000], W.sigs[:12000], W.msgs[:12000], W.pks[:12000])
    bounds = [0, 1, 37, 1000, 4096, 8000, 12000]
    hs = [srv.submit(W.curves[a:b], W.sigs[a:b], W.msgs[a:b], W.pks[a:b]) for a, b in zip(bounds, bounds[1:])]
    for (a, b), h in zip(zip(bounds, bounds[1:]), hs):
        out, st, _ = srv.wait(h)
        assert (out == ref_out[a:b]).all() and (st == ref_st[a:b]).all()
    srv.close()


def test_continuous_batching_needs_no_launch_per_request(w, ref):
    """120 requests submitted back to back are worked off by the running
    kernel: one launch (a relaunch at most if it hits its lifetime)."""
    from wgpu_sig_ops.serving import Server, request_stream

    pool, regions, ref_out, ref_st = ref
    offs, cnts, arr = request_stream(regions, 0.0, 0.0, seed=4, n_requests=120)
    srv = Server(w.default_context(), slots=8, slot_items=32768)
    rc, lat, wall, out, st = srv.run_load(pool, offs, cnts, arr)
    s = srv.stats()
    srv.close()
    assert rc == 0 and (lat > 0).all()
    assert s["requests_done"] == 120 and 1 <= s["launches"] <= 3
    for o, c in zip(offs, cnts):
        sl = slice(int(o), int(o) + int(c))
        assert (out[sl] == ref_out[sl]).all() and (st[sl] == ref_st[sl]).all()


def test_admission_limits(w, W):
    from wgpu_sig_ops._lib import SIGOPS_E_BUSY, SIGOPS_E_RANGE, SigopsError
    from wgpu_sig_ops.serving import Server

    srv = Server(w.default_context(), slots=1, slot_items=1024)
    with pytest.raises(SigopsError) as e:
        srv.submit(W.curves[:2000], W.sigs[:2000], W.msgs[:2000], W.pks[:2000])
    assert e.value.code == SIGOPS_E_RANGE
    # the rings hold one full request: a second one submitted before the
    # first has finished is refused, and fits once it has
    busy = 0
    for _ in range(5):
        h = srv.submit(W.curves[:1024], W.sigs[:1024], W.msgs[:1024], W.pks[:1024])
        try:
            h2 = srv.submit(0, W.sigs[:1], W.msgs[:1])
            srv.wait(h2)
        except SigopsError as e2:
            assert e2.code == SIGOPS_E_BUSY
            busy += 1
        srv.wait(h)
    assert busy >= 1
    h = srv.submit(0, W.sigs[:1], W.msgs[:1])
    out, st, lat = srv.wait(h)
    assert lat > 0
    srv.close()


def test_admission_refuses_below_the_hbm_floor(w, W):
    """With the device's free memory below the floor (1% of the device, at
    least 256 MiB) submits are refused; once it is back they are accepted."""
    torch = pytest.importorskip("torch")
    from wgpu_sig_ops._lib import SIGOPS_E_BUSY, SigopsError
    from wgpu_sig_ops.serving import Server

    srv = Server(w.default_context(), slots=4, slot_items=1024)
    srv.wait(srv.submit(0, W.sigs[:1], W.msgs[:1]))
    free, total = torch.cuda.mem_get_info()
    floor = max(256 << 20, total // 100)
    keep = floor // 2  # left free: below the floor, enough for the runtime
    hog = torch.empty(max(0, free - keep), dtype=torch.uint8, device="cuda") if free > keep else None
    try:
        time.sleep(0.25)  # the dispatcher re-reads free memory every 100 ms
        with pytest.raises(SigopsError) as e:
            srv.submit(0, W.sigs[:1], W.msgs[:1])
        assert e.value.code == SIGOPS_E_BUSY
    finally:
        del hog
        torch.cuda.empty_cache()
    time.sleep(0.25)
    out, st, _ = srv.wait(srv.submit(0, W.sigs[:1], W.msgs[:1]))
    srv.close()


def test_cancel(w, W):
    """A cancelled request's buffers are never written; the handle is released;
    later requests are unaffected.  Cancelling a finished request says so."""
    from wgpu_sig_ops._lib import SIGOPS_E_INVAL, SigopsError, lib
    from wgpu_sig_ops.serving import Server

    srv = Server(w.default_context(), slots=4, slot_items=16384)
    n = 16384
    cur, sig, msg, pk = W.curves[:n], W.sigs[:n], W.msgs[:n], W.pks[:n]
    canceled = 0
    for _ in range(3):
        h = srv.submit(cur, sig, msg, pk)
        bufs = srv._live[h]
        if srv.cancel(h):
            canceled += 1
            # a later request is finished only after the cancelled one's tiles
            out2, st2, _ = srv.wait(srv.submit(cur[:64], sig[:64], msg[:64], pk[:64]))
            assert not bufs[4].any() and not bufs[5].any()
            assert lib.sigops_server_wait(srv.ptr, h, 0, None) == SIGOPS_E_INVAL
        else:
            srv.wait(h)
    assert canceled >= 1
    # cancel after completion: the request counts as done before cancel
    before = srv.stats()["requests_done"]
    h = srv.submit(cur[:8], sig[:8], msg[:8], pk[:8])
    deadline = time.time() + 10
    while srv.stats()["requests_done"] == before and time.time() < deadline:
        time.sleep(0.002)
    assert srv.cancel(h) is False
    out, st, _ = srv.wait(h)
    want_out, want_st = w.batch.verify_mixed(cur[:8], sig[:8], msg[:8], pk[:8])
    assert (out == want_out).all() and (st == want_st).all()
    with pytest.raises(SigopsError) as e:
        srv.cancel(h)
    assert e.value.code == SIGOPS_E_INVAL
    srv.close()


def test_kernel_closes_when_idle_and_relaunches(w, W):
    from wgpu_sig_ops.serving import Server

    srv = Server(w.default_context(), slots=4, slot_items=1024)
    out1, st1, _ = srv.wait(srv.submit(W.curves[:100], W.sigs[:100], W.msgs[:100], W.pks[:100]))
    time.sleep(0.2)  # well past the 20 ms idle close
    out2, st2, _ = srv.wait(srv.submit(W.curves[:100], W.sigs[:100], W.msgs[:100], W.pks[:100]))
    s = srv.stats()
    srv.close()
    assert s["launches"] == 2 and s["requests_done"] == 2
    assert (out1 == out2).all() and (st1 == st2).all()


def test_dispatcher_that_stops(w, W):
    """Host-side failure injection: the dispatcher thread stops as if it had
    died.  Waits end with SIGOPS_E_TIMEDOUT, submits are refused, destroy still
    cleans up, and a new server on the same context works."""
    from wgpu_sig_ops._lib import SIGOPS_E_CUDA, SIGOPS_E_TIMEDOUT, SigopsError
    from wgpu_sig_ops.serving import Server

    ctx = w.default_context()
    srv = Server(ctx, slots=4, slot_items=1024)
    srv.wait(srv.submit(0, W.sigs[:1], W.msgs[:1]))
    srv.test_fault(1)
    time.sleep(0.1)
    try:
        h = srv.submit(0, W.sigs[:4], W.msgs[:4])
        with pytest.raises(SigopsError) as e:
            srv.wait(h, 2000)
        assert e.value.code == SIGOPS_E_TIMEDOUT
    except SigopsError as e:
        assert e.code == SIGOPS_E_CUDA
    srv.close()
    srv2 = Server(ctx, slots=4, slot_items=1024)
    out, st, _ = srv2.wait(srv2.submit(W.curves[:50], W.sigs[:50], W.msgs[:50], W.pks[:50]))
    want_out, want_st = w.batch.verify_mixed(W.curves[:50], W.sigs[:50], W.msgs[:50], W.pks[:50])
    assert (out == want_out).all() and (st == want_st).all()
    srv2.close()


def test_allocation_failures(w, W):
    """Injected allocation failures (on the host, no device fault): a server
    or context that cannot allocate is refused cleanly, a call that cannot
    grow its buffers returns SIGOPS_E_NOMEM, and everything works once
    allocations succeed again."""
    from wgpu_sig_ops._lib import SIGOPS_E_NOMEM, SigopsError, lib
    from wgpu_sig_ops.context import Context
    from wgpu_sig_ops.serving import Server

    ctx = w.default_context()
    try:
        assert lib.sigops_test_fail_allocations(1) == 0
        with pytest.raises(RuntimeError):
            Server(ctx, slots=4, slot_items=1024)
        assert lib.sigops_test_fail_allocations(1) == 0  # the first was used up
        with pytest.raises(RuntimeError):
            Context(0)
        c2 = Context(0)  # the injected failure is used up: this one builds
        n = 3000
        lib.sigops_test_fail_allocations(1)
        with pytest.raises(SigopsError) as e:
            w.batch.verify_mixed(W.curves[:n], W.sigs[:n], W.msgs[:n], W.pks[:n], ctx=c2)
        assert e.value.code == SIGOPS_E_NOMEM
        lib.sigops_test_fail_allocations(0)
        out, st = w.batch.verify_mixed(W.curves[:n], W.sigs[:n], W.msgs[:n], W.pks[:n], ctx=c2)
        want_out, want_st = w.batch.verify_mixed(W.curves[:n], W.sigs[:n], W.msgs[:n], W.pks[:n], ctx=ctx)
        assert (out == want_out).all() and (st == want_st).all()
        c2.close()
    finally:
        lib.sigops_test_fail_allocations(0)


def test_poisson_load_short(w, W):
    from wgpu_sig_ops.serving import measure

    res = measure(w.default_context(), W, loads=(0.5,), seconds=2.0, sat_items=200000, slot_items=16384)
    lvl = res["levels"][0]
    info = ("sat %.3g refused %d rc %d p50 %.3g p99 %.3g gap %.3g drv %.3g launches %d busy %.3g"
            % (res["saturation_sigs_per_s"], lvl["refused"], lvl["rc"], lvl["p50_ms"], lvl["p99_ms"], lvl["dispatch_max_gap_ms"],
               lvl["dispatch_max_driver_ms"], lvl["launches"], lvl["kernel_busy"]))
    assert res["saturation_sigs_per_s"] > 0 and lvl["refused"] == 0 and lvl["p50_ms"] > 0, info
    assert res["stats"]["launches"] >= 1
    ks = res["kernel_stats"]
    assert ks["items"] >= res["stats"]["items_done"] and ks["tiles"] * 32 >= ks["items"] and ks["work_s"] > 0


def test_adaptive_shape(w, ref):
    """With an adaptive shape the server runs the low-latency shape under light
    load, switches to the high-throughput shape while items arrive faster than
    the switch rate, and goes back once the load is gone; every result equals
    the batched engine's."""
    from wgpu_sig_ops.serving import Server, request_stream

    pool, regions, ref_out, ref_st = ref
    # rings for about 0.4 s of the stream below: only the dispatcher thread
    # relaunches the kernel (the shape switch closes it), so the rings must
    # ride out that thread going unscheduled for a while on a busy host
    srv = Server(w.default_context(), slots=256, slot_items=4096)
    srv.set_adaptive(0, 1, 1.0e6)
    sl = slice(0, 100)
    out, st, _ = srv.wait(srv.submit(pool["curves"][sl], pool["sigs"][sl], pool["msgs"][sl], pool["pks"][sl]))
    assert srv.shape_stats()["shape"] == 0
    assert (out == ref_out[sl]).all() and (st == ref_st[sl]).all()
    # 1.5 s of Poisson arrivals at about 2.7M items/s (mean request ~270 items)
    offs, cnts, arr = request_stream(regions, 10000.0, 1.5, seed=9)
    rc, lat, wall, out, st = srv.run_load(pool, offs, cnts, arr)
    busy = srv.shape_stats()
    assert rc == 0 and (lat > 0).all()
    assert busy["switches"] >= 1 and busy["shape"] == 1, busy
    for o, c in zip(offs, cnts):
        s2 = slice(int(o), int(o) + int(c))
        assert (out[s2] == ref_out[s2]).all() and (st[s2] == ref_st[s2]).all()
    # quiet again: the kernel closes when idle, and the next launch takes the low shape
    time.sleep(0.4)
    out, st, _ = srv.wait(srv.submit(pool["curves"][sl], pool["sigs"][sl], pool["msgs"][sl], pool["pks"][sl]))
    quiet = srv.shape_stats()
    srv.close()
    assert quiet["shape"] == 0, quiet
    assert (out == ref_out[sl]).all() and (st == ref_st[sl]).all()
    from wgpu_sig_ops._lib import SIGOPS_E_INVAL, SigopsError

    bad = Server(w.default_context(), slots=2, slot_items=64)
    try:
        for args in ((0, 3, 1.0), (-1, 1, 1.0), (0, 1, 0.0)):
            with pytest.raises(SigopsError) as e:
                bad.set_adaptive(*args)
            assert e.value.code == SIGOPS_E_INVAL
    finally:
        bad.close()
