"""Parity of the CUDA path with the oracle and the golden vectors, through the
drop-in API (the calls a user of the reference makes).  Bit-exact."""
import random

import numpy as np
import pytest

from oracle import sigops_oracle as o
from tests.golden_io import load

pytestmark = pytest.mark.gpu
G = load()
L = 13


@pytest.fixture(scope="module")
def w():
    import wgpu_sig_ops

    return wgpu_sig_ops


def test_k1_reference_kat(w):
    """src/curve_algos/secp256k1_ecdsa.rs:206-214: the signature under secret key 1 recovers G."""
    kat = G["secp256k1_kat"]
    table = w.precompute.secp256k1_bases(L)
    res = w.secp256k1_ecdsa.ecrecover([bytes.fromhex(kat["sig"])], [bytes.fromhex(kat["msg"])], table, L)
    assert res[0].hex() == kat["pubkey"]
    res = w.secp256k1_ecdsa.ecrecover_single_shader([bytes.fromhex(kat["sig"])], [bytes.fromhex(kat["msg"])], L)
    assert res[0].hex() == kat["pubkey"]


@pytest.mark.parametrize("curve", ["secp256k1", "secp256r1"])
@pytest.mark.parametrize("single", [False, True])
def test_ecdsa_golden(w, curve, single):
    mod = getattr(w, curve + "_ecdsa")
    vecs = G[curve] + G[curve + "_edge"]
    sigs = [bytes.fromhex(v["sig"]) for v in vecs]
    msgs = [bytes.fromhex(v["msg"]) for v in vecs]
    if single:
        res = mod.ecrecover_single_shader(sigs, msgs, L)
    else:
        res = mod.ecrecover(sigs, msgs, getattr(w.precompute, curve + "_bases")(L), L)
    _, status = mod.ecrecover_arrays(sigs, msgs, None, L)
    for v, r, st in zip(vecs, res, status):
        assert r.hex() == v["pubkey"], v.get("case")
        assert st == v["status"], v.get("case")


@pytest.mark.parametrize("single", [False, True])
def test_ed25519_golden(w, single):
    vecs = G["ed25519"]
    args = ([bytes.fromhex(v["sig"]) for v in vecs], [bytes.fromhex(v["msg"]) for v in vecs], [bytes.fromhex(v["pubkey"]) for v in vecs])
    if single:
        res = w.ed25519_eddsa.ecverify_single(*args, L)
    else:
        res = w.ed25519_eddsa.ecverify(*args, w.precompute.ed25519_bases(L), L)
    valid, status = w.ed25519_eddsa.ecverify_arrays(*args)
    for v, r, st in zip(vecs, res, status):
        assert r == v["valid"] and st == v["status"], v["case"]


def _ecdsa_batch(curve, n, seed, tamper_no_point=0.0):
    rng = random.Random(seed)
    sigs, msgs = [], []
    for i in range(n):
        d = rng.randrange(1, curve.n)
        msg = rng.randbytes(32)
        sig = o.ecdsa_sign_fuel(curve, d, msg, k=rng.randrange(1, curve.n))
        if rng.random() < tamper_no_point:
            while True:
                x = rng.randrange(1, curve.n)
                if pow((x**3 + curve.a * x + curve.b) % curve.p, (curve.p - 1) // 2, curve.p) == curve.p - 1:
                    break
            sig = x.to_bytes(32, "big") + sig[32:]
        sigs.append(sig)
        msgs.append(msg)
    return sigs, msgs


@pytest.mark.parametrize("curve_name", ["secp256k1", "secp256r1"])
def test_ecdsa_random_batch_vs_oracle(w, curve_name):
    c = o.SECP256K1 if curve_name == "secp256k1" else o.SECP256R1
    sigs, msgs = _ecdsa_batch(c, 700, seed=11, tamper_no_point=0.05)
    keys, status = getattr(w, curve_name + "_ecdsa").ecrecover_arrays(sigs, msgs, None, L)
    for i in range(len(sigs)):
        st, pk = o.ecdsa_recover(c, sigs[i], msgs[i])
        assert status[i] == st
        assert keys[i].tobytes() == (pk if pk else bytes(64))
    assert (status == o.ST_NO_POINT).sum() > 10


@pytest.mark.parametrize("curve_name", ["secp256k1", "secp256r1"])
def test_ecdsa_generator_table_ends(w, curve_name):
    """u1 windows steered to the generator tables' last entries (digits
    +-32768, +-32767 in every window and both GLV halves): the plain kernel
    (drop-in API) and the batched engine against the oracle."""
    from tests.crafted import crafted_signatures

    c = o.SECP256K1 if curve_name == "secp256k1" else o.SECP256R1
    cases = crafted_signatures(c)
    sigs = [s for _, s, _ in cases]
    msgs = [m for _, _, m in cases]
    keys, status = getattr(w, curve_name + "_ecdsa").ecrecover_arrays(sigs, msgs, None, L)
    tag = 0 if curve_name == "secp256k1" else 1
    out, mstatus = w.batch.verify_mixed([tag] * len(cases), sigs, msgs, [bytes(32)] * len(cases))
    for i, (name, sig, msg) in enumerate(cases):
        st, pk = o.ecdsa_recover(c, sig, msg)
        assert st == o.ST_OK, name
        assert (status[i], keys[i].tobytes()) == (st, pk), name
        assert (mstatus[i], bytes(out[i])) == (st, pk), name


def test_ed25519_random_batch_vs_oracle(w):
    rng = random.Random(12)
    sigs, msgs, pks = [], [], []
    for i in range(600):
        seed = rng.randbytes(32)
        msg = o.fuel_message(rng.randbytes(rng.randrange(0, 257)))
        _, _, pk = o.ed25519_keypair(seed)
        sig = o.ed25519_sign(seed, msg)
        mode = rng.randrange(8)
        if mode == 1:
            b = rng.randrange(256)
            sig = bytearray(sig)
            sig[b // 8] ^= 1 << (b % 8)
            sig = bytes(sig)
        elif mode == 2:
            msg = bytes([msg[0] ^ 1]) + msg[1:]
        elif mode == 3:
            sig = sig[:32] + (int.from_bytes(sig[32:], "little") + o.ED_L).to_bytes(32, "little")
        elif mode == 4:
            pk = rng.randbytes(32)
        sigs.append(sig)
        msgs.append(msg)
        pks.append(pk)
    valid, status = w.ed25519_eddsa.ecverify_arrays(sigs, msgs, pks)
    for i in range(len(sigs)):
        st, ok = o.ed25519_ecverify(sigs[i], msgs[i], pks[i])
        assert (status[i], bool(valid[i])) == (st, ok), i


def test_ed25519_raw_golden(w):
    """Messages of any length (0..4096 bytes, around the SHA-512 block
    boundaries of R || A || M) against OpenSSL / libsodium verdicts."""
    from tests.golden_io import load_raw

    V = load_raw()
    valid, status = w.ed25519_eddsa.verify_raw_arrays([bytes.fromhex(v["sig"]) for v in V], [bytes.fromhex(v["msg"]) for v in V],
                                                      [bytes.fromhex(v["pubkey"]) for v in V])
    for k, v in enumerate(V):
        assert bool(valid[k]) == v["valid"], (v["case"], v["len"])
        if v["case"] == "s_plus_l":
            assert status[k] == o.ST_BAD_SCALAR


def test_ed25519_raw_random_vs_oracle(w):
    """Random lengths and tampering, every status equal to the oracle's; the
    32-byte items also equal the fixed-length API."""
    rng = random.Random(31)
    sigs, msgs, pks = [], [], []
    for i in range(400):
        seed = rng.randbytes(32)
        msg = rng.randbytes(rng.choice([0, 1, 32, 47, 48, 111, 112, 175, 176, rng.randrange(0, 700)]))
        _, _, pk = o.ed25519_keypair(seed)
        sig = o.ed25519_sign(seed, msg)
        mode = rng.randrange(6)
        if mode == 1 and msg:
            j = rng.randrange(len(msg))
            msg = msg[:j] + bytes([msg[j] ^ 0x40]) + msg[j + 1:]
        elif mode == 2:
            sig = bytes([sig[0] ^ 1]) + sig[1:]
        elif mode == 3:
            pk = rng.randbytes(32)
        sigs.append(sig)
        msgs.append(msg)
        pks.append(pk)
    valid, status = w.ed25519_eddsa.verify_raw_arrays(sigs, msgs, pks)
    for i in range(len(sigs)):
        st, ok = o.ed25519_verify_raw(sigs[i], msgs[i], pks[i])
        assert (status[i], bool(valid[i])) == (st, ok), (i, len(msgs[i]))
    sel = [i for i in range(len(sigs)) if len(msgs[i]) == 32]
    v32, s32 = w.ed25519_eddsa.ecverify_arrays([sigs[i] for i in sel], [msgs[i] for i in sel], [pks[i] for i in sel])
    assert (v32 == valid[sel]).all() and (s32 == status[sel]).all()


def test_ed25519_raw_bounds(w):
    """A message running past the message buffer is refused on the host."""
    import ctypes

    from wgpu_sig_ops._lib import lib

    seed = bytes(range(32))
    _, _, pk = o.ed25519_keypair(seed)
    sig = o.ed25519_sign(seed, b"abc")
    blob = (ctypes.c_uint8 * 3)(*b"abc")
    offs = (ctypes.c_uint64 * 1)(1)
    lens = (ctypes.c_uint32 * 1)(3)
    valid = (ctypes.c_uint8 * 1)()
    ctx = w.default_context()
    rc = lib.sigops_ed25519_verify_raw(ctx.ptr, sig, blob, 3, offs, lens, pk, 1, valid, None)
    assert rc == -22  # SIGOPS_E_INVAL
    offs[0] = 0
    assert lib.sigops_ed25519_verify_raw(ctx.ptr, sig, blob, 3, offs, lens, pk, 1, valid, None) == 0 and valid[0] == 1


def test_empty_and_errors(w):
    t = w.precompute.secp256k1_bases(L)
    assert w.secp256k1_ecdsa.ecrecover([], [], t, L) == []
    assert w.ed25519_eddsa.ecverify([], [], [], w.precompute.ed25519_bases(L), L) == []
    with pytest.raises(w.SigopsError):
        w.secp256k1_ecdsa.ecrecover([bytes(64)], [bytes(32)], t[:-1], L)
    with pytest.raises(w.SigopsError):
        w.secp256r1_ecdsa.ecrecover([bytes(64)], [bytes(32)], t, L)  # k1 table for r1
    with pytest.raises(ValueError):
        w.secp256k1_ecdsa.ecrecover([bytes(64)], [], t, L)


def test_ragged_sizes(w):
    """Sizes that are not multiples of the block or of a power of two."""
    c = o.SECP256K1
    sigs, msgs = _ecdsa_batch(c, 257, seed=3)
    for n in (1, 2, 31, 33, 255, 257):
        res = w.secp256k1_ecdsa.ecrecover_single_shader(sigs[:n], msgs[:n], L)
        assert res[-1] == o.ecdsa_recover(c, sigs[n - 1], msgs[n - 1])[1]
        assert res[0] == o.ecdsa_recover(c, sigs[0], msgs[0])[1]
