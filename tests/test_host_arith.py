"""The kernels' arithmetic compiled for the host (carry flag emulated), checked
against Python integers, the oracle and the golden vectors.  CPU only."""
import ctypes
import random

import pytest

from oracle import sigops_oracle as o
from tests._paths import build_hostcheck
from tests.golden_io import load

G = load()


@pytest.fixture(scope="module")
def hc():
    return ctypes.CDLL(build_hostcheck())


def le(v):
    return v.to_bytes(32, "little")


MODS = [o.SECP256K1.p, o.SECP256R1.p, o.ED_P, o.SECP256K1.n, o.SECP256R1.n, o.ED_L]


def expected(field, op, a, b):
    m = MODS[field]
    if op == 0:
        return a * b % m
    if op == 1:
        return (a + b) % m
    if op == 2:
        return (a - b) % m
    if op == 3:
        return pow(a, m - 2, m)
    return pow(a, (m + 1) // 4, m) if field < 2 else pow(a, (m - 5) // 8, m)


def test_mul_wide(hc):
    rng = random.Random(5)
    cases = [(2**256 - 1, 2**256 - 1), (0, 5), (2**255, 2)] + [(rng.getrandbits(256), rng.getrandbits(256)) for _ in range(300)]
    for a, b in cases:
        out = ctypes.create_string_buffer(64)
        hc.hc_mul_wide(le(a), le(b), out)
        assert int.from_bytes(out.raw, "little") == a * b


@pytest.mark.parametrize("form", [0, 1], ids=["schoolbook", "karatsuba"])
def test_mul_wide_forms(hc, form):
    """Both 512-bit product forms, including the sign cases of the Karatsuba
    middle term (halves equal, a0 < a1 with b1 < b0, ...) and all-ones limbs."""
    rng = random.Random(50 + form)
    h = 2**128
    cases = [(2**256 - 1, 2**256 - 1), (0, 0), (1, 2**256 - 1), (h, h), (h - 1, h), (h * 5 + 3, h * 3 + 5), (3 * h + 5, 5 * h + 3)]
    for _ in range(400):
        a1, a0, b1, b0 = (rng.choice([rng.getrandbits(128), 0, h - 1, rng.getrandbits(8)]) for _ in range(4))
        cases.append((a1 * h + a0, b1 * h + b0))
    cases += [(rng.getrandbits(256), rng.getrandbits(256)) for _ in range(400)]
    hc.hc_mul_wide_form.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
    for a, b in cases:
        out = ctypes.create_string_buffer(64)
        hc.hc_mul_wide_form(form, le(a), le(b), out)
        assert int.from_bytes(out.raw, "little") == a * b, (hex(a), hex(b))


@pytest.mark.parametrize("field", [0, 1, 2], ids=["k1", "r1", "ed"])
def test_canonical_boundaries(hc, field):
    """Canonicalisation and add/sub next to the reduction boundaries:
    [p, 2^256) for secp256k1 / P-256, and the two ranges around 2^255 for
    ed25519 (before and after folding bit 255)."""
    m = MODS[field]
    xs = [0, 1, m - 1, m, m + 1, 2**256 - 1, 2**256 - 2, 2**255, 2**255 - 1, 2**255 + 18, 2**255 + 19, 2**255 - 19, 2**255 - 20]
    xs += [m + k for k in range(0, 40)] + [2**256 - 1 - k for k in range(0, 40)] + [2**255 + k for k in range(-40, 40)]
    out = ctypes.create_string_buffer(32)
    for x in xs:
        if not 0 <= x < 2**256:
            continue
        hc.hc_canon(field, le(x), out)
        assert int.from_bytes(out.raw, "little") == x % m, hex(x)
    # add / sub with operands next to 0, p and the fold boundaries
    near = [0, 1, 2, 18, 19, 20, 977, 2**32 + 977, m - 1, m - 2, m - 19, m - 20, m // 2, m // 2 + 1, 2**255 - 20 if 2**255 - 20 < m else 5]
    for a in near:
        for b in near:
            for op, f in ((1, lambda a, b: (a + b) % m), (2, lambda a, b: (a - b) % m)):
                hc.hc_field(field, op, le(a), le(b), out)
                assert int.from_bytes(out.raw, "little") == f(a, b), (op, hex(a), hex(b))


# the P-256 field is held in Montgomery form: its reduction returns t 2^-256 mod p
R1_RINV = pow(2**256, -1, o.SECP256R1.p)


def test_p256_reduction(hc):
    """The P-256 Montgomery reduction on products of field elements and on
    extreme 512-bit values (all ones, single high words), where the held-back
    round carries and the final fold reach their bounds: below 2^256 (weakly
    reduced) and equal to t 2^-256 mod p."""
    p = o.SECP256R1.p
    rng = random.Random(70)
    xs = [0, 1, p, p * p, (p - 1) * (p - 1), 2**512 - 1, 2**511, (2**256 - 1) * (2**256 - 1)]
    xs += [sum(rng.choice([0, 0xFFFFFFFF, 1, 0x80000000]) << (32 * k) for k in range(16)) for _ in range(300)]
    xs += [rng.randrange(p) * rng.randrange(p) for _ in range(300)] + [rng.getrandbits(512) for _ in range(300)]
    out = ctypes.create_string_buffer(32)
    for x in xs:
        hc.hc_r1_reduce(x.to_bytes(64, "little"), out)
        r = int.from_bytes(out.raw, "little")
        assert r < 2**256 and r % p == x * R1_RINV % p, hex(x)


def test_sqr_wide(hc):
    rng = random.Random(6)
    cases = [2**256 - 1, 0, 1, 2**255, 2**32 - 1] + [rng.getrandbits(256) for _ in range(500)]
    cases += [sum(rng.choice([0, 0xFFFFFFFF]) << (32 * k) for k in range(8)) for _ in range(100)]
    for a in cases:
        out = ctypes.create_string_buffer(64)
        hc.hc_sqr_wide(le(a), out)
        assert int.from_bytes(out.raw, "little") == a * a, hex(a)


@pytest.mark.parametrize("field", range(6))
@pytest.mark.parametrize("op", range(5))
def test_field_ops(hc, field, op):
    if op == 4 and field > 2:
        pytest.skip("no root / p58 power in scalar fields")
    m = MODS[field]
    rng = random.Random(field * 10 + op)
    cases = [(m - 1, m - 1), (0, m - 1), (1, 1), (m - 1, 1)] + [(rng.randrange(m), rng.randrange(m)) for _ in range(60)]
    for a, b in cases:
        out = ctypes.create_string_buffer(32)
        hc.hc_field(field, op, le(a), le(b), out)
        assert int.from_bytes(out.raw, "little") == expected(field, op, a, b), (field, op, hex(a), hex(b))


def test_sha512(hc):
    for v in G["sha512_96"]:
        out = ctypes.create_string_buffer(64)
        hc.hc_sha512_96(bytes.fromhex(v["in"]), out)
        assert out.raw.hex() == v["out"]


@pytest.mark.parametrize("curve", ["secp256k1", "secp256k1_glv", "secp256r1"])
def test_ecdsa_golden(hc, curve):
    fn = {"secp256k1": hc.hc_k1_recover, "secp256k1_glv": hc.hc_k1_recover_glv, "secp256r1": hc.hc_r1_recover}[curve]
    curve = curve.replace("_glv", "")
    for v in G[curve] + G[curve + "_edge"]:
        out = ctypes.create_string_buffer(64)
        st = fn(bytes.fromhex(v["sig"]), bytes.fromhex(v["msg"]), out)
        want = bytes.fromhex(v["pubkey"]) if v["pubkey"] else bytes(64)
        assert (st, out.raw) == (v["status"], want), v.get("case")


def test_k1_kat(hc):
    kat = G["secp256k1_kat"]
    out = ctypes.create_string_buffer(64)
    assert hc.hc_k1_recover(bytes.fromhex(kat["sig"]), bytes.fromhex(kat["msg"]), out) == 0
    assert out.raw.hex() == kat["pubkey"]


def test_ed25519_golden(hc):
    for v in G["ed25519"]:
        st = hc.hc_ed_verify(bytes.fromhex(v["sig"]), bytes.fromhex(v["msg"]), bytes.fromhex(v["pubkey"]))
        assert st == v["status"], v["case"]


def test_ed25519_raw_golden(hc):
    """Messages of any length: the multi-block challenge hash straddles the
    SHA-512 block boundaries; verdicts from OpenSSL and libsodium."""
    from tests.golden_io import load_raw

    hc.hc_ed_verify_raw.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_char_p]
    for v in load_raw():
        m = bytes.fromhex(v["msg"])
        st = hc.hc_ed_verify_raw(bytes.fromhex(v["sig"]), m, len(m), bytes.fromhex(v["pubkey"]))
        assert (st == 0) == v["valid"], (v["case"], v["len"])


def test_random_vs_oracle(hc):
    rng = random.Random(77)
    for i in range(12):
        d = rng.randrange(1, o.SECP256R1.n)
        msg = rng.randbytes(32)
        for c, fn in ((o.SECP256K1, hc.hc_k1_recover), (o.SECP256R1, hc.hc_r1_recover)):
            sig = o.ecdsa_sign_fuel(c, d % c.n or 1, msg)
            out = ctypes.create_string_buffer(64)
            st = fn(sig, msg, out)
            assert (st, out.raw) == (0, o.ws_public_key(c, d % c.n or 1))
        seed = rng.randbytes(32)
        _, _, pk = o.ed25519_keypair(seed)
        sig = o.ed25519_sign(seed, msg)
        assert hc.hc_ed_verify(sig, msg, pk) == 0


def test_kernel_tables(hc):
    """The device tables hold (i+1)*G for every entry (affine, in the field's
    representation: integers for secp256k1, Montgomery form for P-256); the
    secp256k1 table continues with (i+1)*2^128*G (GLV)."""
    ne, ned = hc.hc_gtab_entries(0), hc.hc_gtab_entries(1)
    assert ne == ned == 1 << 15  # generator windows of 16 bits
    for curve, c, halves in ((0, o.SECP256K1, 2), (1, o.SECP256R1, 1)):
        buf = (ctypes.c_uint32 * (halves * ne * 16))()
        hc.hc_gtab(curve, buf)
        words = buf
        for h in range(halves):
            for i in (0, 1, 15, 255, 256, 4097, ne - 2, ne - 1):
                e = h * ne + i
                x = sum(words[e * 16 + k] << (32 * k) for k in range(8))
                y = sum(words[e * 16 + 8 + k] << (32 * k) for k in range(8))
                if curve == 1:
                    x, y = x * R1_RINV % c.p, y * R1_RINV % c.p
                assert (x, y) == o.ws_mul(c, (i + 1) << (128 * h), c.g), (curve, h, i)
    buf = (ctypes.c_uint32 * (ned * 24))()
    hc.hc_gtab(2, buf)
    words = buf
    for i in (0, 7, 255, 256, 9999, ned - 1):
        x, y = o.ed_mul(i + 1, o.ED_B)
        ypx = sum(words[i * 24 + k] << (32 * k) for k in range(8))
        ymx = sum(words[i * 24 + 8 + k] << (32 * k) for k in range(8))
        assert ypx == (x + y) % o.ED_P and ymx == (y - x) % o.ED_P


@pytest.mark.parametrize("curve", [0, 1, 2])
def test_bases_bit_identical(hc, curve):
    fn = [o.secp256k1_bases, o.secp256r1_bases, o.ed25519_bases][curve]
    for L in range(11, 16):
        exp = fn(L)
        buf = (ctypes.c_uint32 * len(exp))()
        assert hc.hc_bases(curve, L, buf) == len(exp)
        assert list(buf) == exp


def test_signers_match_oracle(hc):
    rng = random.Random(9)
    for i in range(12):
        m = rng.randbytes(32)
        for cid, c in ((0, o.SECP256K1), (1, o.SECP256R1)):
            d, k = rng.randrange(1, c.n), rng.randrange(1, c.n)
            sig, pub = ctypes.create_string_buffer(64), ctypes.create_string_buffer(64)
            assert hc.hc_ecdsa_sign(cid, d.to_bytes(32, "big"), k.to_bytes(32, "big"), m, sig, pub) == 0
            assert sig.raw == o.ecdsa_sign_fuel(c, d, m, k=k)
            assert pub.raw == o.ws_public_key(c, d)
        seed = rng.randbytes(32)
        sig, pk = ctypes.create_string_buffer(64), ctypes.create_string_buffer(32)
        hc.hc_ed_sign(seed, m, sig, pk)
        assert sig.raw == o.ed25519_sign(seed, m)
        assert pk.raw == o.ed25519_keypair(seed)[2]


def test_k1_glv_vs_oracle(hc):
    """GLV path (batched engine) on random signatures, scalar edge cases and the
    Strauss edge case of the reference's tests."""
    rng = random.Random(31)
    c = o.SECP256K1
    for i in range(60):
        d = rng.randrange(1, c.n) if i > 3 else [1, 2, c.n - 1, c.n // 2][i]
        msg = rng.randbytes(32) if i % 5 else (c.n - 1).to_bytes(32, "big")
        sig = o.ecdsa_sign_fuel(c, d, msg, k=rng.randrange(1, c.n))
        out = ctypes.create_string_buffer(64)
        st = hc.hc_k1_recover_glv(sig, msg, out)
        assert (st, out.raw) == o.ecdsa_recover(c, sig, msg)[0:1] + (o.ecdsa_recover(c, sig, msg)[1] or bytes(64),)


@pytest.mark.parametrize("field", [0, 1, 2], ids=["secp256k1", "secp256r1", "ed25519"])
def test_reduce_512(hc, field):
    """Reduction of 512-bit values, including those whose folds carry out of
    2^256 again (low half near 2^256, high half extreme): below 2^256, equal
    mod p (P-256: equal to x 2^-256 mod p, its Montgomery reduction)."""
    p = [o.SECP256K1.p, o.SECP256R1.p, o.ED_P][field]
    top = 2**256
    rng = random.Random(90 + field)
    highs = [0, 1, 2**32 - 1, 2**32, top - 1, top - 2, 2**255, 2**224, top - 2**32, 2**64 - 1]
    lows = [0, 1, top - 1, top - 2, top - 977, top - 2**32 - 977, top - 38, top - 39, top - 2**33, top - 2**66, top - 2**70]
    xs = [h * top + l for h in highs for l in lows]
    xs += [rng.getrandbits(256) * top + (top - rng.getrandbits(rng.choice([8, 40, 70, 100]))) for _ in range(400)]
    xs += [rng.getrandbits(512) for _ in range(400)]
    if field != 1:
        # the first fold L + H (2^256 - p) lands just below a multiple of 2^256,
        # so that folding its top words carries out again
        c = top - p if field == 0 else 38
        for _ in range(400):
            h = rng.getrandbits(256)
            delta = rng.randrange(1, 2**rng.choice([4, 10, 20, 40, 64]))
            l = (top - delta - h * c) % top
            xs.append(h * top + l)
    out = ctypes.create_string_buffer(32)
    for x in xs:
        hc.hc_reduce(field, x.to_bytes(64, "little"), out)
        r = int.from_bytes(out.raw, "little")
        assert r < top and r % p == (x * R1_RINV if field == 1 else x) % p, hex(x)


@pytest.mark.parametrize("field", [0, 1, 2], ids=["secp256k1", "secp256r1", "ed25519"])
def test_weak_reduction(hc, field):
    """The three base fields keep values below 2^256 only: add /
    sub / mul / sqr / neg on inputs anywhere in [0, 2^256), including the
    double-carry and double-borrow corrections, stay below 2^256 and agree mod
    p; is_zero recognises both representations of zero."""
    top = 2**256
    if field == 0:
        p = o.SECP256K1.p
        c = top - p  # 2^32 + 977
        edge = [0, 1, 976, 977, 978, c - 1, c, c + 1, 2 * c, p - 1, p, p + 1, p + c - 1, 2**255, top - 1, top - 2, top - c, top - c - 1,
                top - c + 1, top - 2 * c, 2**32, 2**64 - 1]
        for v, z in ((0, 1), (p, 1), (1, 0), (p - 1, 0), (p + 1, 0), (top - 1, 0)):
            out = ctypes.create_string_buffer(32)
            hc.hc_weak(0, 5, le(v), le(0), out)
            assert out.raw[0] == z, hex(v)
    elif field == 1:
        p = o.SECP256R1.p
        k = top - p
        edge = [0, 1, 2, k - 1, k, k + 1, 2 * k, p - 1, p, p + 1, p + k - 1, 2**255, top - 1, top - 2, top - k, top - k - 1, top - k + 1,
                2**224, 2**192, 2**96, 2**96 - 1, top - 2**224]
        for v, z in ((0, 1), (p, 1), (1, 0), (p - 1, 0), (p + 1, 0), (top - 1, 0)):
            out = ctypes.create_string_buffer(32)
            hc.hc_weak(1, 5, le(v), le(0), out)
            assert out.raw[0] == z, hex(v)
    else:
        p = o.ED_P
        edge = [0, 1, 18, 19, 37, 38, 39, p - 1, p, p + 1, p + 37, 2**255, top - 1, top - 2, top - 37, top - 38, top - 39, top - 76]
    rng = random.Random(41 + field)
    vals = edge + [rng.getrandbits(256) for _ in range(30)]
    mscale = R1_RINV if field == 1 else 1  # P-256 multiplies in Montgomery form
    for a in vals:
        for b in vals:
            ops = [(0, lambda a, b: a + b), (1, lambda a, b: a - b), (2, lambda a, b: a * b * mscale), (3, lambda a, b: a * a * mscale),
                   (4, lambda a, b: -a)]
            if field < 2:
                ops.append((6, lambda a, b: a * pow(2, -1, p)))
            for op, f in ops:
                if op >= 3 and b != vals[0]:
                    continue
                out = ctypes.create_string_buffer(32)
                hc.hc_weak(field, op, le(a), le(b), out)
                r = int.from_bytes(out.raw, "little")
                assert r < top and r % p == f(a, b) % p, (op, hex(a), hex(b))


def test_generator_table_ends(hc):
    """Recovery with u1 windows steered to the generator tables' last entries
    (digits +-32768, +-32767, every window, both GLV halves), host build of
    the plain and GLV kernels against the oracle."""
    from tests.crafted import crafted_signatures

    for c, fns in ((o.SECP256K1, (hc.hc_k1_recover, hc.hc_k1_recover_glv)), (o.SECP256R1, (hc.hc_r1_recover,))):
        for name, sig, msg in crafted_signatures(c):
            st, pk = o.ecdsa_recover(c, sig, msg)
            assert st == o.ST_OK, name
            for fn in fns:
                out = ctypes.create_string_buffer(64)
                assert (fn(sig, msg, out), out.raw) == (st, pk), name


@pytest.mark.parametrize("name", ["k1p", "k1n", "r1p", "r1n", "edp", "edl"])
def test_divstep_inverse(hc, name):
    """Bernstein-Yang divstep inverse (20 batches of 30 half-delta divsteps):
    exact against pow() without the Fermat fallback, and every input reaches
    g = 0 within the fixed batch count."""
    M, minv = {"k1p": (o.SECP256K1.p, 0x2ddacacf), "k1n": (o.SECP256K1.n, 0x2a774ec1), "r1p": (o.SECP256R1.p, 0x3fffffff),
               "r1n": (o.SECP256R1.n, 0x11ff43b1), "edp": (o.ED_P, 0x179435e5), "edl": (o.ED_L, 0x2dab81e5)}[name]
    assert pow(M, -1, 2**30) == minv
    rng = random.Random(hash(name) & 0xffff)
    cases = [1, 2, 3, M - 1, M - 2, (M - 1) // 2, 2**255 % M, 2**128] + [rng.randrange(1, M) for _ in range(3000)]
    for x in cases:
        out = ctypes.create_string_buffer(32)
        used = ctypes.c_int()
        hc.hc_divstep_inv(x.to_bytes(32, "little"), M.to_bytes(32, "little"), minv, out, ctypes.byref(used))
        assert int.from_bytes(out.raw, "little") == pow(x, -1, M)
        assert 0 < used.value <= 20


@pytest.mark.parametrize("curve", [0, 1], ids=["secp256k1", "secp256r1"])
def test_weierstrass_exceptional_cases(hc, curve):
    """Jacobian add / mixed add / double against the oracle, including the
    exceptional inputs the Strauss loop can meet: P + P (falls back to
    doubling), P + (-P) = infinity, infinity + Q, P + infinity, and points
    with non-unit, different Z."""
    c = o.SECP256K1 if curve == 0 else o.SECP256R1
    rng = random.Random(90 + curve)
    hc.hc_weier_op.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_char_p] * 5
    G = c.g

    def pt(k):
        return o.ws_mul(c, k, G)

    def enc(A):
        return le(A[0]) + le(A[1]) if A is not None else bytes(64)

    def run(op, A, za, B, zb):
        out = ctypes.create_string_buffer(64)
        inf = hc.hc_weier_op(curve, op, enc(A), le(za if A is not None else 0), enc(B), le(zb if B is not None else 0), out)
        return None if inf else (int.from_bytes(out.raw[:32], "little"), int.from_bytes(out.raw[32:], "little"))

    def add_ref(A, B):
        return o._to_affine(c, o._jac_add(c, None if A is None else (A[0], A[1], 1), None if B is None else (B[0], B[1], 1)))

    cases = []
    for _ in range(12):
        A, B = pt(rng.randrange(1, c.n)), pt(rng.randrange(1, c.n))
        negA = (A[0], (-A[1]) % c.p)
        cases += [(A, B), (A, A), (A, negA), (None, B), (A, None), (None, None)]
    for A, B in cases:
        za, zb = rng.randrange(1, c.p), rng.randrange(1, c.p)
        assert run(0, A, za, B, zb) == add_ref(A, B)
        if B is not None:  # mixed add: Q affine, never infinity
            assert run(1, A, za, B, 1) == add_ref(A, B)
        assert run(2, A, za, None, 0) == add_ref(A, A)


@pytest.mark.parametrize("curve", [0, 1, 2], ids=["secp256k1", "secp256r1", "ed25519"])
@pytest.mark.parametrize("batch", [1, 3, 16])
def test_batched_shared_inversions(hc, curve, batch):
    """The batched engine's single-curve path (r^-1 and the result's Z^-1 by
    simultaneous inversion over a thread's items), host build, on golden and
    tampered items: every record and status equals the oracle's, including
    threads whose items all fail (nothing to invert) and sizes that leave the
    last threads short."""
    from tests.golden_io import load

    G2 = load()
    name = ["secp256k1", "secp256r1", "ed25519"][curve]
    vecs = G2[name] + (G2.get(name + "_edge", []) if curve < 2 else [])
    sigs = b"".join(bytes.fromhex(v["sig"]) for v in vecs)
    msgs = b"".join(bytes.fromhex(v["msg"]) for v in vecs)
    pks = b"".join(bytes.fromhex(v["pubkey"]) if curve == 2 else bytes(32) for v in vecs)
    n = len(vecs)
    for m in (n, 1, 17, min(n, 33)):
        out = ctypes.create_string_buffer(64 * m)
        st = ctypes.create_string_buffer(m)
        hc.hc_batched_deferred(curve, sigs[:64 * m], msgs[:32 * m], pks[:32 * m], ctypes.c_size_t(m), batch, out, st)
        for k in range(m):
            v = vecs[k]
            if curve == 2:
                exp = bytes([1 if v["valid"] else 0]) + bytes(63)
            else:
                exp = bytes.fromhex(v["pubkey"]) if v["pubkey"] else bytes(64)
            assert (out.raw[64 * k:64 * k + 64], st.raw[k]) == (exp, v["status"]), (m, k)


def test_coz_table_iso(hc):
    """The inversion-free secp256k1 table of R multiples: each entry at the
    chain's last Z equals the affine entry mapped to the isomorphic curve,
    (x zc^2, y zc^3), for the generator, its negation and random points."""
    hc.hc_coz_iso_mismatches.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    c = o.SECP256K1
    rng = random.Random(17)
    points = [c.g, (c.g[0], c.p - c.g[1])]
    while len(points) < 40:
        x = rng.randrange(1, c.p)
        rhs = (x * x * x + c.b) % c.p
        y = pow(rhs, (c.p + 1) // 4, c.p)
        if y * y % c.p == rhs:
            points.append((x, y))
    for x, y in points:
        assert hc.hc_coz_iso_mismatches(le(x), le(y)) == 0, (hex(x), hex(y))
