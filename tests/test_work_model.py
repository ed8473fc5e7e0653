"""The committed work model (multiply instructions per signature, the
roofline numerator) matches what the current kernel source issues."""
import json
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_work_model_is_current():
    from tests.hostcheck import work_model

    with open(work_model.OUT) as f:
        committed = json.load(f)
    fresh = work_model.compute()
    for key in ("secp256k1_glv", "secp256k1", "secp256r1", "ed25519", "mul_wide", "sqr_wide"):
        assert committed[key] == pytest.approx(fresh[key], rel=1e-12), key
    assert committed["phases"] == fresh["phases"]
    # the product forms: schoolbook 64 x (lo + hi); squaring 36 x (lo + hi)
    assert fresh["mul_wide"] == 128 and fresh["sqr_wide"] == 72
