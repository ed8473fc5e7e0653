"""The autotuner: times every launch variant on a device-signed probe batch,
applies the fastest, stores it in the cache file and sigops_create reads it
back; results are unchanged by the choice."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_selects_and_caches(tmp_path, monkeypatch):
    import wgpu_sig_ops as w
    from wgpu_sig_ops import workload as wl

    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("SIGOPS_TUNE_CACHE", str(cache))
    ctx = w.Context(0)
    W = wl.config("c4", n=4000, seed=12, ctx=ctx)
    before = w.batch.verify_mixed(W.curves, W.sigs, W.msgs, W.pks, ctx=ctx)
    rep = ctx.autotune(probe_items=152 * 256)
    assert len(rep["chosen"]) == 4 and "batched" in rep
    # per curve: every configuration timed, with its launch shape and window widths
    for curve in ("secp256k1", "secp256r1", "ed25519"):
        cfgs = rep["curve_configs"][curve]
        assert len(cfgs) == 8
        assert {c["wr"] for c in cfgs.values()} == {4, 5, 6} and {c["wg"] for c in cfgs.values()} == {8, 16}
        assert {c["block"] for c in cfgs.values()} == {64, 128, 256, 512}
    v = ctx.variants()
    assert [v[k]["variant"] for k in ("plain_secp256k1", "plain_secp256r1", "plain_ed25519", "batched")] == rep["chosen"]
    after = w.batch.verify_mixed(W.curves, W.sigs, W.msgs, W.pks, ctx=ctx)
    assert (before[0] == after[0]).all() and (before[1] == after[1]).all()
    assert cache.exists() and cache.read_text().strip()
    ctx2 = w.Context(0)  # reads the cache
    v2 = ctx2.variants()
    assert [v2[k]["variant"] for k in ("plain_secp256k1", "plain_secp256r1", "plain_ed25519", "batched")] == rep["chosen"]
    ctx2.close()
    ctx.close()
