"""The benchmark configurations at full size: bit-exact against the C oracle
(c1 1,024 secp256k1; c2 65,536 ed25519 with 3% tampered; c3 262,144 P-256
with 1% r that has no curve point), and the 1,048,576-item mixed batch through
generator-known outcomes, plain == batched, and the C oracle on every one of
its items."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def w():
    import wgpu_sig_ops

    return wgpu_sig_ops


def _oracle(curve, W):
    from oracle import c_oracle

    return c_oracle.batch(curve, W.sigs, W.msgs, W.pks if curve == 2 else None)


def test_c1_secp256k1_1024(w):
    from wgpu_sig_ops import workload as wl

    W = wl.config("c1")
    keys, st = w.secp256k1_ecdsa.ecrecover_arrays(W.sigs, W.msgs, w.precompute.secp256k1_bases(13), 13)
    o_keys, o_st = _oracle(0, W)
    assert (st == o_st).all() and (keys == o_keys).all()
    assert (keys == W.expect_key).all()


def test_c2_ed25519_65536(w):
    from wgpu_sig_ops import workload as wl

    W = wl.config("c2")
    valid, st = w.ed25519_eddsa.ecverify_arrays(W.sigs, W.msgs, W.pks, w.precompute.ed25519_bases(13), 13)
    o_valid, o_st = _oracle(2, W)
    assert (st == o_st).all() and (valid == o_valid).all()
    assert int((valid == 0).sum()) == int((W.tamper != 0).sum()) == round(0.03 * 65536)


def test_c3_secp256r1_262144(w):
    from wgpu_sig_ops import workload as wl

    W = wl.config("c3")
    keys, st = w.secp256r1_ecdsa.ecrecover_arrays(W.sigs, W.msgs, w.precompute.secp256r1_bases(13), 13)
    o_keys, o_st = _oracle(1, W)
    assert (st == o_st).all() and (keys == o_keys).all()
    assert int((st == 2).sum()) == round(0.01 * 262144)
    # the Vec<u8> view: empty exactly where the oracle errs
    vecs = w.secp256r1_ecdsa.ecrecover(W.sigs[:4096], W.msgs[:4096], w.precompute.secp256r1_bases(13), 13)
    assert [len(v) for v in vecs] == [64 if s == 0 else 0 for s in o_st[:4096]]


def test_c4_mixed_1m(w):
    from oracle import c_oracle
    from wgpu_sig_ops import workload as wl

    W = wl.config("c4")
    out, st = w.batch.verify_mixed(W.curves, W.sigs, W.msgs, W.pks)
    chk = wl.expected_check(W, out, st)
    assert chk["mismatches"] == 0, chk
    # plain per-curve kernels give the same bytes
    for c, mod in ((0, w.secp256k1_ecdsa), (1, w.secp256r1_ecdsa)):
        sel = np.nonzero(W.curves == c)[0][:50000]
        keys, s2 = mod.ecrecover_arrays(W.sigs[sel], W.msgs[sel])
        assert (keys == out[sel]).all() and (s2 == st[sel]).all()
    # the C oracle on all 1,048,576 items (all host threads)
    o_out, o_st = c_oracle.batch_mixed(W.curves, W.sigs, W.msgs, W.pks)
    bad = np.nonzero((o_st != st) | (o_out != out).any(axis=1))[0]
    assert len(bad) == 0, f"{len(bad)} items differ from the oracle, first {bad[:5].tolist()}"
