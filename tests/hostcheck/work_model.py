#!/usr/bin/env python
"""Work model of the kernels: 32-bit multiply instructions per signature.

The host build of the kernels' own source (tests/hostcheck) counts every
multiply its carry-chain primitives issue (a 32x32 -> 64-bit product is two:
low half and high half) plus the wide products of the divstep inverse.  The
count of one signature is fixed by the algorithm (fixed windows, fixed
addition chains, fixed divstep count); it is averaged over the valid golden
vectors of each path.  bench.py divides it, times signatures per second, by
the measured rate of the same instruction form (sigops_probe_mul form 2).

    python tests/hostcheck/work_model.py            # prints the model
    python tests/hostcheck/work_model.py --write    # and stores profiles/work_model.json
"""
from __future__ import annotations

import ctypes
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.join(ROOT, "profiles", "work_model.json")


def compute() -> dict:
    sys.path.insert(0, ROOT)
    from tests._paths import build_hostcheck

    hc = ctypes.CDLL(build_hostcheck())
    hc.hc_mulcount.restype = ctypes.c_uint64
    hc.hc_mulcount.argtypes = [ctypes.c_int]
    with open(os.path.join(ROOT, "tests", "golden", "vectors.json")) as f:
        G = json.load(f)

    def per_sig(fn, items, args):
        total = 0
        for v in items:
            hc.hc_mulcount(1)
            st = fn(*args(v))
            assert st == 0, "work model uses valid signatures only"
            total += hc.hc_mulcount(1)
        return total / len(items)

    out = ctypes.create_string_buffer(64)

    def ecdsa_args(v):
        return bytes.fromhex(v["sig"]), bytes.fromhex(v["msg"]), out

    k1 = [v for v in G["secp256k1"] if v["status"] == 0]
    r1 = [v for v in G["secp256r1"] if v["status"] == 0]
    ed = [v for v in G["ed25519"] if v["status"] == 0]
    hc.hc_k1_recover(*ecdsa_args(k1[0]))  # builds the generator tables outside the count
    model = {
        "unit": "32-bit multiply instructions per signature (lo and hi halves counted separately)",
        "source": "host build of the kernel source (tests/hostcheck), averaged over the valid golden vectors",
        "secp256k1_glv": per_sig(hc.hc_k1_recover_glv, k1, ecdsa_args),
        "secp256k1": per_sig(hc.hc_k1_recover, k1, ecdsa_args),
        "secp256r1": per_sig(hc.hc_r1_recover, r1, ecdsa_args),
        "ed25519": per_sig(hc.hc_ed_verify, ed, lambda v: (bytes.fromhex(v["sig"]), bytes.fromhex(v["msg"]), bytes.fromhex(v["pubkey"]))),
        "samples": {"secp256k1": len(k1), "secp256r1": len(r1), "ed25519": len(ed)},
    }
    # the batched engine's single-curve path: r^-1 and Z^-1 by simultaneous
    # inversion over 16 items per thread (its INV_BATCH), counted per item
    def per_sig_batched(curve, items):
        n = len(items)
        sigs = b"".join(bytes.fromhex(v["sig"]) for v in items)
        msgs = b"".join(bytes.fromhex(v["msg"]) for v in items)
        pks = b"".join(bytes.fromhex(v["pubkey"]) if curve == 2 else bytes(32) for v in items)
        o = ctypes.create_string_buffer(64 * n)
        st = ctypes.create_string_buffer(n)
        hc.hc_mulcount(1)
        hc.hc_batched_deferred(curve, sigs, msgs, pks, ctypes.c_size_t(n), 16, o, st)
        assert st.raw == bytes(n), "work model uses valid signatures only"
        return hc.hc_mulcount(1) / n

    model["batched"] = {"secp256k1_glv": per_sig_batched(0, k1), "secp256r1": per_sig_batched(1, r1), "ed25519": per_sig_batched(2, ed),
                        "inv_batch": 16}
    # multiplies of the phases whose count does not depend on the batch: one
    # inversion (divsteps, result checked by one multiplication) and one square
    # root chain per field, less the conversions in and out of the field's
    # representation that hc_field adds around every operation
    x = (12345678901234567890).to_bytes(32, "little")

    def op_count(field, op):
        hc.hc_mulcount(1)
        hc.hc_field(field, op, x, x, out)
        n = hc.hc_mulcount(1)
        hc.hc_field(field, 1, x, x, out)  # an addition: the conversions only
        return n - hc.hc_mulcount(1)

    def raw_count(field, op):
        hc.hc_mulcount(1)
        hc.hc_field(field, op, x, x, out)
        return hc.hc_mulcount(1)

    phases = {"fp_inv": {}, "sqrt": {}, "scalar_inv": {}}
    for c, name in ((0, "secp256k1"), (1, "secp256r1"), (2, "ed25519")):
        phases["fp_inv"][name] = op_count(c, 3)
        phases["sqrt"][name] = op_count(c, 4)
    for c, name in ((0, "secp256k1"), (1, "secp256r1")):
        phases["scalar_inv"][name] = raw_count(3 + c, 5)  # r^-1 as the kernels compute it (no conversions around it)
    model["phases"] = phases
    a = bytes(range(32))
    hc.hc_mulcount(1)
    hc.hc_sqr_wide(a, out)
    model["sqr_wide"] = hc.hc_mulcount(1)
    hc.hc_mul_wide(a, a, out)
    model["mul_wide"] = hc.hc_mulcount(1)
    return model


if __name__ == "__main__":
    m = compute()
    print(json.dumps(m, indent=1))
    if "--write" in sys.argv:
        with open(OUT, "w") as f:
            json.dump(m, f, indent=1)
            f.write("\n")
