"""Continuous-batching serving loop (``sigops_server_*`` in libsigops.so).

``Server`` queues verification requests.  Submit copies a request into
pinned, mapped request rings and cuts it into 32-item single-curve tiles; one
persistent kernel, resident on every SM, pulls published tiles into a
device-resident tile ring and works them off, so requests that arrive while
others run cost no launch and no host round trip.  A native dispatcher thread
copies finished requests' results out and relaunches the kernel after it
closes (20 ms idle or 2 s of life).  ``measure`` drives the serving
benchmark: saturation throughput first (a closed backlog), then Poisson
arrivals at fractions of it, reporting throughput and p50 / p99 / p99.9
request latency per load level.
"""

from __future__ import annotations

import ctypes

import numpy as np

from ._batch import ptr
from ._lib import SIGOPS_ALREADY_DONE, SIGOPS_OK, check, lib

_u64p = ctypes.POINTER(ctypes.c_uint64)
_dblp = ctypes.POINTER(ctypes.c_double)


class Server:
    """slot_items: the largest request (0 = 16,384); slots x slot_items items
    may be in flight.  variant: shape of the persistent kernel, 0 = 256-thread
    blocks one per SM, 1 = 128 x 3 per SM, 2 = 256 x 2 per SM."""

    def __init__(self, ctx, slots: int = 32, slot_items: int = 0, hbm_fraction: float = 0.25, variant: int | None = None):
        self.ctx = ctx
        self.ptr = lib.sigops_server_create(ctx.ptr, slots, slot_items, hbm_fraction)
        if not self.ptr:
            raise RuntimeError("sigops_server_create failed")
        self.slot_items = lib.sigops_server_slot_items(self.ptr)
        self._live = {}
        if variant is not None:
            self.set_variant(variant)

    def set_variant(self, variant: int):
        """Shape of the persistent kernel (0..2), from its next launch on."""
        check(lib.sigops_server_set_variant(self.ptr, variant), "sigops_server_set_variant")

    def set_adaptive(self, low_shape: int, high_shape: int, switch_items_per_s: float):
        """Each launch takes high_shape while items arrive at switch_items_per_s
        or more, low_shape below 80% of it."""
        check(lib.sigops_server_set_adaptive(self.ptr, low_shape, high_shape, float(switch_items_per_s)), "sigops_server_set_adaptive")

    def shape_stats(self) -> dict:
        """Shape of the running (or last) launch, adaptive switches, arrival rate."""
        sh, sw, r = ctypes.c_int(), ctypes.c_uint64(), ctypes.c_double()
        check(lib.sigops_server_shape_stats(self.ptr, ctypes.byref(sh), ctypes.byref(sw), ctypes.byref(r)), "sigops_server_shape_stats")
        return {"shape": sh.value, "switches": sw.value, "items_per_s": r.value}

    def submit(self, curves, sigs: np.ndarray, msgs: np.ndarray, pks: np.ndarray | None = None) -> int:
        """Queue one request; ``curves`` is an array of tags or a single curve id."""
        sigs = np.ascontiguousarray(sigs, dtype=np.uint8).reshape(-1, 64)
        msgs = np.ascontiguousarray(msgs, dtype=np.uint8).reshape(-1, 32)
        n = len(sigs)
        if pks is not None:
            pks = np.ascontiguousarray(pks, dtype=np.uint8).reshape(-1, 32)
        cur = None
        uniform = -1
        if np.isscalar(curves):
            uniform = int(curves)
        else:
            cur = np.ascontiguousarray(curves, dtype=np.uint8)
        out = np.zeros((n, 64), np.uint8)
        status = np.zeros(n, np.uint8)
        h = ctypes.c_uint64()
        check(lib.sigops_server_submit(self.ptr, ptr(cur) if cur is not None else None, uniform, ptr(sigs), ptr(msgs),
                                       ptr(pks) if pks is not None else None, n, ptr(out), ptr(status), ctypes.byref(h)),
              "sigops_server_submit")
        self._live[h.value] = (cur, sigs, msgs, pks, out, status)  # keep buffers alive
        return h.value

    def wait(self, handle: int, timeout_ms: int = -1):
        """Returns (out, status, latency_ms)."""
        lat = ctypes.c_double()
        check(lib.sigops_server_wait(self.ptr, handle, timeout_ms, ctypes.byref(lat)), "sigops_server_wait")
        bufs = self._live.pop(handle)
        return bufs[4], bufs[5], lat.value

    def cancel(self, handle: int) -> bool:
        """Withdraw a request.  True when it was cancelled (its buffers are
        released), False when it had already finished (wait() returns it)."""
        rc = lib.sigops_server_cancel(self.ptr, handle)
        if rc == SIGOPS_OK:
            self._live.pop(handle, None)
            return True
        if rc == SIGOPS_ALREADY_DONE:
            return False
        check(rc, "sigops_server_cancel")
        return False

    def kernel_stats(self) -> dict:
        """Counters of the persistent kernel: tiles, items, warp-seconds working
        and looking for work, and the busy fraction."""
        t, i, mv = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        w, d = ctypes.c_double(), ctypes.c_double()
        check(lib.sigops_server_kernel_stats(self.ptr, ctypes.byref(t), ctypes.byref(i), ctypes.byref(w), ctypes.byref(d),
                                             ctypes.byref(mv)), "sigops_server_kernel_stats")
        tot = w.value + d.value
        return {"tiles": t.value, "items": i.value, "work_s": w.value, "idle_s": d.value, "sm_moves": mv.value,
                "busy_fraction": w.value / tot if tot > 0 else 0.0}

    def dispatch_stats(self) -> dict:
        """Dispatcher iterations, the longest gap between two of them with
        requests in flight and its longest driver call, since the previous
        call (ms)."""
        it, gap, drv = ctypes.c_uint64(), ctypes.c_double(), ctypes.c_double()
        check(lib.sigops_server_dispatch_stats(self.ptr, ctypes.byref(it), ctypes.byref(gap), ctypes.byref(drv)),
              "sigops_server_dispatch_stats")
        return {"iterations": it.value, "max_gap_ms": gap.value, "max_driver_ms": drv.value}

    def test_fault(self, fault: int):
        """Failure injection on the host (1: the dispatcher thread stops)."""
        check(lib.sigops_server_test_fault(self.ptr, fault), "sigops_server_test_fault")

    def stats(self) -> dict:
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        q = ctypes.c_size_t()
        check(lib.sigops_server_stats(self.ptr, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(q)), "stats")
        return {"launches": a.value, "requests_done": b.value, "items_done": c.value, "queued_items": q.value}

    def run_load(self, pool: dict, offsets: np.ndarray, counts: np.ndarray, arrivals: np.ndarray):
        """Open-loop run over a pool (dict of curves/sigs/msgs/pks arrays).
        Returns (latency_ms array, wall seconds, out, status)."""
        n = len(pool["curves"])
        # written (not just allocated) here, so that their first-touch page
        # faults do not land in the server's completion path during the run
        out = np.empty((n, 64), np.uint8)
        out.fill(0)
        status = np.empty(n, np.uint8)
        status.fill(0)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        counts = np.ascontiguousarray(counts, dtype=np.uint32)
        arrivals = np.ascontiguousarray(arrivals, dtype=np.float64)
        lat = np.zeros(len(offsets), np.float64)
        wall = ctypes.c_double()
        rc = lib.sigops_server_run_load(self.ptr, ptr(pool["curves"]), ptr(pool["sigs"]), ptr(pool["msgs"]), ptr(pool["pks"]),
                                        ptr(offsets), ptr(counts), ptr(arrivals), len(offsets), ptr(out), ptr(status), ptr(lat),
                                        ctypes.byref(wall))
        return rc, lat, wall.value, out, status

    def close(self):
        if self.ptr:
            lib.sigops_server_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def curve_sorted_pool(W) -> tuple[dict, dict]:
    """Items of a workload grouped by curve (contiguous region per curve)."""
    order = np.argsort(W.curves, kind="stable")
    pool = {"curves": np.ascontiguousarray(W.curves[order]), "sigs": np.ascontiguousarray(W.sigs[order]),
            "msgs": np.ascontiguousarray(W.msgs[order]), "pks": np.ascontiguousarray(W.pks[order]), "src": order}
    regions = {}
    for c in (0, 1, 2):
        idx = np.nonzero(pool["curves"] == c)[0]
        regions[c] = (int(idx[0]), int(len(idx))) if len(idx) else (0, 0)
    return pool, regions


def request_stream(regions: dict, rate_rps: float, seconds: float, seed: int, max_size: int = 2048, mix=(0.4, 0.3, 0.3),
                   n_requests: int | None = None):
    """Poisson arrivals (rate_rps requests/s for `seconds`, or n_requests at
    time 0 when rate_rps is 0) of single-curve requests with sizes
    floor(exp(U(0, ln max_size))) and curves drawn 40/30/30."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if rate_rps > 0:
        gaps = rng.exponential(1.0 / rate_rps, size=int(rate_rps * seconds * 1.2) + 16)
        arrivals = np.cumsum(gaps)
        arrivals = arrivals[arrivals < seconds]
    else:
        arrivals = np.zeros(n_requests)
    m = len(arrivals)
    curves = rng.choice(3, size=m, p=np.array(mix) / np.sum(mix))
    sizes = np.floor(np.exp(rng.uniform(0.0, np.log(max_size), size=m))).astype(np.int64)
    sizes = np.clip(sizes, 1, max_size)
    offsets = np.zeros(m, np.uint64)
    for c in (0, 1, 2):
        sel = np.nonzero(curves == c)[0]
        start, length = regions[c]
        sizes[sel] = np.minimum(sizes[sel], max(1, length))
        offsets[sel] = start + rng.integers(0, np.maximum(1, length - sizes[sel] + 1))
    return offsets, sizes.astype(np.uint32), arrivals


def measure(ctx, W, loads=(0.25, 0.5, 0.75, 0.9), seconds: float = 10.0, seed: int = 5001, slots: int = 0,
            slot_items: int = 0, sat_items: int = 2_000_000, variant: int | None = None, warmup_seconds: float = 1.0,
            adaptive: tuple | None = None) -> dict:
    """Saturation, a discarded warm-up run at half load, then open-loop Poisson
    load levels; latency percentiles in ms.  slots = 0 sizes the request rings
    to hold the whole saturation backlog (plus 10%), and at least 1M items
    (about 50 ms of work at saturation, 200 MB of pinned memory).  adaptive:
    (low_shape, high_shape, switch_items_per_s) for Server.set_adaptive, set
    after the saturation run, which runs high_shape (the shape a sustained
    overload gets)."""
    pool, regions = curve_sorted_pool(W)
    per = slot_items or 16384
    if slots <= 0:
        slots = max(int(np.ceil(1_048_576 / per)), int(np.ceil(1.1 * sat_items / per)))
    if adaptive is not None:
        variant = adaptive[1]
    srv = Server(ctx, slots=slots, slot_items=slot_items, variant=variant)
    try:
        mean_size = float(np.mean(np.clip(np.floor(np.exp(np.random.default_rng(1).uniform(0, np.log(2048), 200000))), 1, 2048)))
        # the backlog must fit the rings, or its tail is refused
        cap_items = 0.9 * slots * srv.slot_items
        n_sat = max(64, int(min(sat_items, cap_items) / mean_size))
        offs, cnts, arr = request_stream(regions, 0.0, 0.0, seed, n_requests=n_sat)
        rc, lat, wall, out, st = srv.run_load(pool, offs, cnts, arr)
        check(rc, "saturation run")
        sat = float(cnts[lat >= 0].sum()) / wall
        res = {"saturation_sigs_per_s": sat, "mean_request_items": mean_size, "slot_items": srv.slot_items, "slots": slots, "kernel_shape": 0 if variant is None else variant,
               "seconds_per_level": seconds, "warmup_seconds": warmup_seconds, "levels": []}
        if adaptive is not None:
            res["adaptive"] = {"low_shape": adaptive[0], "high_shape": adaptive[1], "switch_items_per_s": float(adaptive[2])}
            srv.set_adaptive(*adaptive)
        if warmup_seconds > 0:  # an open-loop run at half load whose latencies are discarded
            offs, cnts, arr = request_stream(regions, 0.5 * sat / mean_size, warmup_seconds, seed + 100)
            check(srv.run_load(pool, offs, cnts, arr)[0], "warm-up run")
        for k, load in enumerate(loads):
            rate = load * sat / mean_size
            offs, cnts, arr = request_stream(regions, rate, seconds, seed + 1 + k)
            k0 = srv.kernel_stats()
            srv.dispatch_stats()
            sh0 = srv.shape_stats()
            rc, lat, wall, out, st = srv.run_load(pool, offs, cnts, arr)
            k1 = srv.kernel_stats()
            dsp = srv.dispatch_stats()
            sh1 = srv.shape_stats()
            ok = lat >= 0
            work, idle, tiles = k1["work_s"] - k0["work_s"], k1["idle_s"] - k0["idle_s"], k1["tiles"] - k0["tiles"]
            res["levels"].append({
                "load": load, "offered_sigs_per_s": float(cnts.sum()) / seconds, "achieved_sigs_per_s": float(cnts[ok].sum()) / wall,
                "requests": int(len(lat)), "refused": int((~ok).sum()),
                "p50_ms": float(np.percentile(lat[ok], 50)), "p99_ms": float(np.percentile(lat[ok], 99)),
                "p999_ms": float(np.percentile(lat[ok], 99.9)), "rc": int(rc),
                "kernel_busy": work / (work + idle) if work + idle > 0 else 0.0,
                "warp_ms_per_tile": 1e3 * work / tiles if tiles else 0.0, "sm_moves": k1["sm_moves"] - k0["sm_moves"],
                "dispatch_max_gap_ms": dsp["max_gap_ms"], "dispatch_max_driver_ms": dsp["max_driver_ms"],
                "launches": srv.stats()["launches"], "shape_at_end": sh1["shape"], "shape_switches": sh1["switches"] - sh0["switches"]})
        res["stats"] = srv.stats()
        res["kernel_stats"] = srv.kernel_stats()
        return res
    finally:
        srv.close()
