"""Continuous-batching serving loop (``sigops_server_*`` in libsigops.so).

``Server`` queues verification requests; a native dispatcher thread keeps
several batches in flight and packs requests that arrive meanwhile into the
next free slot.  ``measure`` drives the serving benchmark: saturation
throughput first (a closed backlog), then Poisson arrivals at fractions of it,
reporting throughput and p50 / p99 / p99.9 request latency per load level.
"""

from __future__ import annotations

import ctypes

import numpy as np

from ._batch import ptr
from ._lib import check, lib

_u64p = ctypes.POINTER(ctypes.c_uint64)
_dblp = ctypes.POINTER(ctypes.c_double)


class Server:
    def __init__(self, ctx, slots: int = 8, slot_items: int = 0, hbm_fraction: float = 0.25, variant: int | None = None):
        self.ctx = ctx
        self.ptr = lib.sigops_server_create(ctx.ptr, slots, slot_items, hbm_fraction)
        if not self.ptr:
            raise RuntimeError("sigops_server_create failed")
        self.slot_items = lib.sigops_server_slot_items(self.ptr)
        self._live = {}
        if variant is not None:
            self.set_variant(variant)

    def set_variant(self, variant: int):
        """Batched-engine launch variant of the server's launches (next launch on)."""
        check(lib.sigops_server_set_variant(self.ptr, variant), "sigops_server_set_variant")

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


def measure(ctx, W, loads=(0.25, 0.5, 0.75, 0.9), seconds: float = 10.0, seed: int = 5001, slots: int = 8,
            slot_items: int = 0, sat_items: int = 2_000_000, variant: int | None = None, warmup_seconds: float = 1.0) -> dict:
    """Saturation, a discarded warm-up run at half load, then open-loop Poisson
    load levels; latency percentiles in ms."""
    pool, regions = curve_sorted_pool(W)
    srv = Server(ctx, slots=slots, slot_items=slot_items, variant=variant)
    try:
        mean_size = float(np.mean(np.clip(np.floor(np.exp(np.random.default_rng(1).uniform(0, np.log(2048), 200000))), 1, 2048)))
        n_sat = max(64, int(sat_items / mean_size))
        offs, cnts, arr = request_stream(regions, 0.0, 0.0, seed, n_requests=n_sat)
        rc, lat, wall, out, st = srv.run_load(pool, offs, cnts, arr)
        check(rc, "saturation run")
        sat = float(cnts.sum()) / wall
        res = {"saturation_sigs_per_s": sat, "mean_request_items": mean_size, "slot_items": srv.slot_items, "slots": slots, "variant": 1 if variant is None else variant,
               "seconds_per_level": seconds, "warmup_seconds": warmup_seconds, "levels": []}
        if warmup_seconds > 0:  # an open-loop run at half load whose latencies are discarded
            offs, cnts, arr = request_stream(regions, 0.5 * sat / mean_size, warmup_seconds, seed + 100)
            check(srv.run_load(pool, offs, cnts, arr)[0], "warm-up run")
        for k, load in enumerate(loads):
            rate = load * sat / mean_size
            offs, cnts, arr = request_stream(regions, rate, seconds, seed + 1 + k)
            rc, lat, wall, out, st = srv.run_load(pool, offs, cnts, arr)
            ok = lat >= 0
            res["levels"].append({
                "load": load, "offered_sigs_per_s": float(cnts.sum()) / seconds, "achieved_sigs_per_s": float(cnts[ok].sum()) / wall,
                "requests": int(len(lat)), "refused": int((~ok).sum()),
                "p50_ms": float(np.percentile(lat[ok], 50)), "p99_ms": float(np.percentile(lat[ok], 99)),
                "p999_ms": float(np.percentile(lat[ok], 99.9)), "rc": int(rc)})
        res["stats"] = srv.stats()
        return res
    finally:
        srv.close()
