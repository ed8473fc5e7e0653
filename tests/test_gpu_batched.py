"""The batched mixed-curve engine: parity with the oracle and with the plain
per-curve kernels, CUDA-graph plans, ragged sizes."""
import random

import numpy as np
import pytest

from oracle import sigops_oracle as o
from tests.golden_io import load

pytestmark = pytest.mark.gpu
G = load()


@pytest.fixture(scope="module")
def w():
    import wgpu_sig_ops

    return wgpu_sig_ops


def golden_mixed(seed=0):
    """All golden vectors of the three curves, shuffled into one batch."""
    items = []
    for curve, tag in (("secp256k1", 0), ("secp256r1", 1)):
        for v in G[curve] + G[curve + "_edge"]:
            exp = bytes.fromhex(v["pubkey"]) if v["pubkey"] else bytes(64)
            items.append((tag, bytes.fromhex(v["sig"]), bytes.fromhex(v["msg"]), bytes(32), exp, v["status"]))
    for v in G["ed25519"]:
        exp = bytes([1 if v["valid"] else 0]) + bytes(63)
        items.append((2, bytes.fromhex(v["sig"]), bytes.fromhex(v["msg"]), bytes.fromhex(v["pubkey"]), exp, v["status"]))
    random.Random(seed).shuffle(items)
    return items


def test_golden_mixed(w):
    items = golden_mixed()
    out, status = w.batch.verify_mixed([i[0] for i in items], [i[1] for i in items], [i[2] for i in items], [i[3] for i in items])
    for k, it in enumerate(items):
        assert out[k].tobytes() == it[4] and status[k] == it[5], (k, it[0])


def oracle_mixed(items):
    res = []
    for tag, sig, msg, pk in items:
        if tag == 2:
            st, ok = o.ed25519_ecverify(sig, msg, pk)
            res.append((bytes([int(ok)]) + bytes(63), st))
        else:
            st, key = o.ecdsa_recover(o.SECP256K1 if tag == 0 else o.SECP256R1, sig, msg)
            res.append((key or bytes(64), st))
    return res


def random_items(n, seed):
    rng = random.Random(seed)
    items = []
    for i in range(n):
        tag = rng.choice([0, 0, 1, 2])
        msg = rng.randbytes(32)
        if tag == 2:
            seed_b = rng.randbytes(32)
            _, _, pk = o.ed25519_keypair(seed_b)
            sig = o.ed25519_sign(seed_b, msg)
            if rng.random() < 0.1:
                sig = sig[:32] + (int.from_bytes(sig[32:], "little") + o.ED_L).to_bytes(32, "little")
            items.append((2, sig, msg, pk))
        else:
            c = o.SECP256K1 if tag == 0 else o.SECP256R1
            sig = o.ecdsa_sign_fuel(c, rng.randrange(1, c.n), msg, k=rng.randrange(1, c.n))
            if rng.random() < 0.1:
                sig = rng.randbytes(32) + sig[32:]  # r replaced: mostly no point or a different key
            items.append((tag, sig, msg, bytes(32)))
    return items


def test_random_mixed_vs_oracle(w):
    items = random_items(600, seed=21)
    out, status = w.batch.verify_mixed(*zip(*items))
    for k, (exp, st) in enumerate(oracle_mixed(items)):
        assert out[k].tobytes() == exp and status[k] == st, k


@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 257])
def test_ragged_sizes(w, n):
    items = random_items(n, seed=100 + n)
    out, status = w.batch.verify_mixed(*zip(*items))
    for k, (exp, st) in enumerate(oracle_mixed(items)):
        assert out[k].tobytes() == exp and status[k] == st, k


def test_single_curve_batches(w):
    for tag in (0, 1, 2):
        items = [it for it in random_items(200, seed=7 + tag) if it[0] == tag] or random_items(1, seed=1)
        out, status = w.batch.verify_mixed(*zip(*items))
        for k, (exp, st) in enumerate(oracle_mixed(items)):
            assert out[k].tobytes() == exp and status[k] == st


def test_matches_plain_kernels(w):
    items = random_items(300, seed=33)
    out, status = w.batch.verify_mixed(*zip(*items))
    for tag, mod in ((0, w.secp256k1_ecdsa), (1, w.secp256r1_ecdsa)):
        sel = [k for k, it in enumerate(items) if it[0] == tag]
        keys, st = mod.ecrecover_arrays([items[k][1] for k in sel], [items[k][2] for k in sel])
        assert (keys == out[sel]).all() and (st == status[sel]).all()
    sel = [k for k, it in enumerate(items) if it[0] == 2]
    valid, st = w.ed25519_eddsa.ecverify_arrays([items[k][1] for k in sel], [items[k][2] for k in sel], [items[k][3] for k in sel])
    assert (valid == out[sel, 0]).all() and (st == status[sel]).all()


# single-curve variant 4 + a + 8 b + 64 c: each curve in every one of its eight
# configurations (launch shapes, per-point windows 4 / 5 / 6, generator
# windows 16 / 8 with the table staged into shared memory)
SPLIT = [4 + k + 8 * ((k + 1) % 8) + 64 * ((k + 2) % 8) for k in range(8)]


@pytest.mark.parametrize("variant", [0, 1, 2, 3] + SPLIT)
def test_every_launch_variant(w, variant):
    """Fused (0..3) and single-curve (4..515) variants give the oracle's
    results, on a mixed batch and on ragged ones that leave some curves
    empty."""
    ctx = w.Context(0)
    ctx.set_variant(3, variant)
    assert ctx.variants()["batched"]["variant"] == variant
    for n, seed in ((400, 61), (1, 62), (33, 63)):
        items = random_items(n, seed=seed)
        out, status = w.batch.verify_mixed(*zip(*items), ctx=ctx)
        for k, (exp, st) in enumerate(oracle_mixed(items)):
            assert out[k].tobytes() == exp and status[k] == st, (variant, n, k)
    ctx.close()


@pytest.mark.parametrize("variant", [0, 515])
def test_graph_plan_replays(w, variant):
    import torch

    from wgpu_sig_ops._lib import check, lib

    ctx = w.Context(0)
    ctx.set_variant(3, variant)
    items = random_items(200, seed=44)
    ref_out, ref_st = w.batch.verify_mixed(*zip(*items))
    cur, sig, msg, pk = zip(*items)
    d_cur = torch.tensor(cur, dtype=torch.uint8, device="cuda")
    d_sig = torch.from_numpy(np.frombuffer(b"".join(sig), np.uint8).copy()).cuda()
    d_msg = torch.from_numpy(np.frombuffer(b"".join(msg), np.uint8).copy()).cuda()
    d_pk = torch.from_numpy(np.frombuffer(b"".join(pk), np.uint8).copy()).cuda()
    d_out = torch.zeros((len(items), 64), dtype=torch.uint8, device="cuda")
    d_st = torch.full((len(items),), 9, dtype=torch.uint8, device="cuda")
    plan = w.batch.MixedPlan(ctx, d_cur.data_ptr(), d_sig.data_ptr(), d_msg.data_ptr(), d_pk.data_ptr(), len(items), d_out.data_ptr(),
                             d_st.data_ptr())
    for _ in range(3):
        d_out.zero_()
        torch.cuda.synchronize()
        plan.launch()
        check(lib.sigops_sync(ctx.ptr), "sync")
        assert (d_out.cpu().numpy() == ref_out).all() and (d_st.cpu().numpy() == ref_st).all()
    plan.close()
    ctx.close()


def test_rejects_bad_curve_tag(w):
    with pytest.raises(w.SigopsError):
        w.batch.verify_mixed([3], [bytes(64)], [bytes(32)], [bytes(32)])
    out, st = w.batch.verify_mixed([], [], [], [])
    assert out.shape == (0, 64)


def test_workload_generator_selfcheck(w):
    """The device signer + tamper generator agrees with the batched engine."""
    from wgpu_sig_ops import workload as wl

    W = wl.config("c4", n=8192, seed=5)
    out, status = w.batch.verify_mixed(W.curves, W.sigs, W.msgs, W.pks)
    chk = wl.expected_check(W, out, status)
    assert chk["mismatches"] == 0, chk
    # and a sample against the oracle
    idx = np.random.default_rng(0).choice(W.n, 200, replace=False)
    items = [(int(W.curves[i]), W.sigs[i].tobytes(), W.msgs[i].tobytes(), W.pks[i].tobytes()) for i in idx]
    for k, (exp, st) in enumerate(oracle_mixed(items)):
        assert out[idx[k]].tobytes() == exp and status[idx[k]] == st


def test_pipelined_host_call(w):
    """Page-locked calls of 131,072 items or more run as two halves on two
    streams; the results match the generator-known outcomes and the
    single-stream device call, at an odd size that splits off-centre."""
    import torch
    from wgpu_sig_ops import workload as wl

    W = wl.config("c4", n=200003, seed=9)
    ctx = w.default_context()
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    h_out = torch.zeros((W.n, 64), dtype=torch.uint8).pin_memory().numpy()
    h_st = torch.full((W.n,), 0xFF, dtype=torch.uint8).pin_memory().numpy()
    w.batch.verify_mixed_into(ctx, pin(W.curves), pin(W.sigs), pin(W.msgs), pin(W.pks), h_out, h_st)
    chk = wl.expected_check(W, h_out, h_st)
    assert chk["mismatches"] == 0, chk
    out, status = w.batch.verify_mixed(W.curves, W.sigs, W.msgs, W.pks)  # staged, one stream
    assert (out == h_out).all() and (status == h_st).all()
