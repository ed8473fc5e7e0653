"""Failure detection without a GPU fault: a bounded wait that runs out (an
mbarrier nothing arrives on) is reported as SIGOPS_E_TIMEDOUT through the
device error word, and the context keeps working afterwards."""
import pytest

from oracle import sigops_oracle as o

pytestmark = pytest.mark.gpu


def test_wait_expiry_is_reported_and_context_survives():
    import wgpu_sig_ops as w
    from wgpu_sig_ops._lib import lib

    ctx = w.Context(0)
    for _ in range(2):  # the error word is cleared after each report
        assert lib.sigops_test_wait_expiry(ctx.ptr, 1000) == -110  # SIGOPS_E_TIMEDOUT
        assert b"wait expired" in lib.sigops_last_error()
    assert lib.sigops_test_wait_expiry(ctx.ptr, 0) == -22  # out-of-range poll count refused on the host
    c = o.SECP256K1
    d, m = 0x1234567, bytes(range(32))
    sig = o.ecdsa_sign_fuel(c, d, m)
    keys = w.secp256k1_ecdsa.ecrecover([sig], [m], w.precompute.secp256k1_bases(13), 13, ctx=ctx)
    assert keys == [o.ws_public_key(c, d)]
    ctx.sync()
    ctx.close()
