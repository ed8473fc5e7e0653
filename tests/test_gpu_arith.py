"""Device arithmetic (field ops, wide product, SHA-512) against Python integers."""
import random

import numpy as np
import pytest

from tests.golden_io import load
from tests.test_host_arith import MODS, expected

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import wgpu_sig_ops as w

    return w.default_context()


def run_field(ctx, field, op, pairs):
    import ctypes

    from wgpu_sig_ops._lib import check, lib

    n = len(pairs)
    a = b"".join(x.to_bytes(32, "little") for x, _ in pairs)
    b = b"".join(y.to_bytes(32, "little") for _, y in pairs)
    out = ctypes.create_string_buffer(64 * n)
    check(lib.sigops_test_field(ctx.ptr, field, op, a, b, out, n), "sigops_test_field")
    raw = out.raw
    return [int.from_bytes(raw[64 * i:64 * i + 64], "little") for i in range(n)]


def test_mul_wide(ctx):
    rng = random.Random(3)
    pairs = [(2**256 - 1, 2**256 - 1), (0, 1)] + [(rng.getrandbits(256), rng.getrandbits(256)) for _ in range(2000)]
    got = run_field(ctx, 0, 5, pairs)
    assert got == [a * b for a, b in pairs]


@pytest.mark.parametrize("field", range(6))
@pytest.mark.parametrize("op", range(5))
def test_field_ops(ctx, field, op):
    if op == 4 and field > 2:
        pytest.skip("no root / p58 power in scalar fields")
    m = MODS[field]
    rng = random.Random(100 + field * 10 + op)
    pairs = [(m - 1, m - 1), (0, m - 1), (1, 1), (m - 1, 1), (2**128, 2**128)] + [(rng.randrange(m), rng.randrange(m)) for _ in range(1000)]
    got = run_field(ctx, field, op, pairs)
    for (a, b), g in zip(pairs, got):
        assert g % 2**256 == expected(field, op, a, b), (field, op, hex(a), hex(b))


def test_sha512(ctx):
    import ctypes

    from wgpu_sig_ops._lib import check, lib

    vecs = load()["sha512_96"]
    inp = b"".join(bytes.fromhex(v["in"]) for v in vecs)
    out = ctypes.create_string_buffer(64 * len(vecs))
    check(lib.sigops_test_sha512(ctx.ptr, inp, out, len(vecs)), "sigops_test_sha512")
    for i, v in enumerate(vecs):
        assert out.raw[64 * i:64 * i + 64].hex() == v["out"]


def test_imad_probe(ctx):
    rate = ctx.probe_imad()
    assert 1e12 < rate < 1e14
