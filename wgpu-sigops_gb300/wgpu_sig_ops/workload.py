"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: keys, nonces, seeds and messages come from
``numpy.random.Generator(PCG64(seed))``, and the signatures are made on the
GPU by ``sigops_workload_sign_*`` (low-s fuel encodings for ECDSA, RFC 8032 for
ed25519), then a seeded fraction is tampered on the host.

Each generated item carries its expected outcome, so a run can check itself
without an oracle:

* untampered ECDSA items recover the signer's public key;
* ``no_point``: r replaced by an x with no curve point -> status NO_POINT;
* ``flip_msg`` (ECDSA): one message bit flipped -> status OK, another key;
* ed25519 ``flip_R`` / ``flip_msg`` -> MISMATCH, ``s_plus_l`` -> BAD_SCALAR.

Configurations (sizes, mixes and tamper rates of the benchmark suite):
  c1: 1,024 secp256k1 recoveries
  c2: 65,536 ed25519 verifications, 3% tampered (R bit, message bit, S+l)
  c3: 262,144 P-256 recoveries, 1% r with no curve point
  c4: 1,048,576 mixed 40/30/30, requests log-uniform in 1..4096 interleaved,
      2% tampered
"""

from __future__ import annotations

import hashlib
from dataclasses import dataclass, field

import numpy as np

from ._lib import ED25519, SECP256K1, SECP256R1, check, lib

# curve orders and field primes (for tampering on the host)
N = {
    SECP256K1: 0xFFFFFFFFFFFFFFFFFFFFFFFFFFFFFFFEBAAEDCE6AF48A03BBFD25E8CD0364141,
    SECP256R1: 0xFFFFFFFF00000000FFFFFFFFFFFFFFFFBCE6FAADA7179E84F3B9CAC2FC632551,
}
P = {SECP256K1: 2**256 - 2**32 - 977, SECP256R1: 2**256 - 2**224 + 2**192 + 2**96 - 1}
AB = {SECP256K1: (0, 7), SECP256R1: (-3, 0x5AC635D8AA3A93E7B3EBBD55769886BC651D06B0CC53B0F63BCE3C3E27D2604B)}
ED_L = 2**252 + 27742317777372353535851937790883648493

# tamper codes
T_NONE, T_NO_POINT, T_FLIP_MSG, T_FLIP_R, T_S_PLUS_L = 0, 1, 2, 3, 4


@dataclass
class Workload:
    name: str
    curves: np.ndarray  # (n,) uint8
    sigs: np.ndarray  # (n, 64) uint8
    msgs: np.ndarray  # (n, 32) uint8
    pks: np.ndarray  # (n, 32) uint8 (ed25519 keys; zero for ECDSA items)
    expect_key: np.ndarray  # (n, 64) uint8: signer's key for ECDSA items
    tamper: np.ndarray  # (n,) uint8 tamper code
    requests: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))  # request sizes in order

    @property
    def n(self) -> int:
        return len(self.curves)

    def counts(self) -> dict:
        return {int(c): int((self.curves == c).sum()) for c in (SECP256K1, SECP256R1, ED25519)}

    def subset(self, idx: np.ndarray, name: str | None = None) -> "Workload":
        return Workload(name or self.name, self.curves[idx], self.sigs[idx], self.msgs[idx], self.pks[idx],
                        self.expect_key[idx], self.tamper[idx])


def _torch():
    import torch

    return torch


def _sign_ecdsa(ctx, curve: int, secrets: np.ndarray, nonces: np.ndarray, msgs: np.ndarray):
    torch = _torch()
    n = len(secrets)
    dev = torch.device("cuda")
    d_s = torch.from_numpy(secrets).to(dev)
    d_k = torch.from_numpy(nonces).to(dev)
    d_m = torch.from_numpy(msgs).to(dev)
    d_sig = torch.empty((n, 64), dtype=torch.uint8, device=dev)
    d_pub = torch.empty((n, 64), dtype=torch.uint8, device=dev)
    d_st = torch.empty(n, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    check(lib.sigops_workload_sign_ecdsa(ctx.ptr, curve, d_s.data_ptr(), d_k.data_ptr(), d_m.data_ptr(), n, d_sig.data_ptr(),
                                         d_pub.data_ptr(), d_st.data_ptr(), stream or None), "sigops_workload_sign_ecdsa")
    check(lib.sigops_sync(ctx.ptr), "sigops_sync")
    return d_sig.cpu().numpy(), d_pub.cpu().numpy(), d_st.cpu().numpy()


def _sign_ed(ctx, seeds: np.ndarray, msgs: np.ndarray):
    torch = _torch()
    n = len(seeds)
    dev = torch.device("cuda")
    d_sd = torch.from_numpy(seeds).to(dev)
    d_m = torch.from_numpy(msgs).to(dev)
    d_sig = torch.empty((n, 64), dtype=torch.uint8, device=dev)
    d_pk = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    check(lib.sigops_workload_sign_ed25519(ctx.ptr, d_sd.data_ptr(), d_m.data_ptr(), n, d_sig.data_ptr(), d_pk.data_ptr(), None),
          "sigops_workload_sign_ed25519")
    check(lib.sigops_sync(ctx.ptr), "sigops_sync")
    return d_sig.cpu().numpy(), d_pk.cpu().numpy()


def _no_point_x(rng: np.random.Generator, curve: int) -> int:
    p, n = P[curve], N[curve]
    a, b = AB[curve]
    while True:
        x = int.from_bytes(rng.bytes(32), "big") % n
        if x == 0:
            continue
        rhs = (x * x * x + a * x + b) % p
        if pow(rhs, (p - 1) // 2, p) == p - 1:
            return x


def make(n_by_curve: dict, seed: int, tamper_rate: dict, ctx=None, ed_raw_len=(0, 256), name="custom",
         curves_order: np.ndarray | None = None, ecdsa_modes=(T_NO_POINT, T_FLIP_MSG)) -> Workload:
    """Generate signatures for the given per-curve counts.  ``tamper_rate`` maps
    curve -> fraction; ``curves_order`` (optional) gives the final item order
    as curve tags (items of one curve appear in generation order)."""
    from .context import default_context

    ctx = ctx or default_context()
    rng = np.random.Generator(np.random.PCG64(seed))
    parts = {}
    for curve in (SECP256K1, SECP256R1):
        m = n_by_curve.get(curve, 0)
        if not m:
            continue
        secrets = rng.integers(0, 256, size=(m, 32), dtype=np.uint8)
        nonces = rng.integers(0, 256, size=(m, 32), dtype=np.uint8)
        msgs = rng.integers(0, 256, size=(m, 32), dtype=np.uint8)
        for _ in range(8):
            sigs, pubs, st = _sign_ecdsa(ctx, curve, secrets, nonces, msgs)
            bad = np.nonzero(st)[0]
            if not len(bad):
                break
            secrets[bad] = rng.integers(0, 256, size=(len(bad), 32), dtype=np.uint8)
            nonces[bad] = rng.integers(0, 256, size=(len(bad), 32), dtype=np.uint8)
        else:
            raise RuntimeError("signing kept failing")
        tam = np.zeros(m, np.uint8)
        k = int(round(m * tamper_rate.get(curve, 0.0)))
        if k:
            sel = rng.choice(m, size=k, replace=False)
            for j, i in enumerate(sel):
                if ecdsa_modes[j % len(ecdsa_modes)] == T_NO_POINT:
                    x = _no_point_x(rng, curve)
                    sigs[i, :32] = np.frombuffer(x.to_bytes(32, "big"), np.uint8)
                    tam[i] = T_NO_POINT
                else:
                    bit = int(rng.integers(0, 256))
                    msgs[i, bit // 8] ^= np.uint8(1 << (bit % 8))
                    tam[i] = T_FLIP_MSG
        parts[curve] = (sigs, msgs, np.zeros((m, 32), np.uint8), pubs, tam)
    m = n_by_curve.get(ED25519, 0)
    if m:
        seeds = rng.integers(0, 256, size=(m, 32), dtype=np.uint8)
        lens = rng.integers(ed_raw_len[0], ed_raw_len[1] + 1, size=m)
        raws = [rng.bytes(int(L)) for L in lens]
        msgs = np.frombuffer(b"".join(hashlib.sha256(r).digest() for r in raws), np.uint8).reshape(m, 32).copy()
        sigs, pks = _sign_ed(ctx, seeds, msgs)
        tam = np.zeros(m, np.uint8)
        k = int(round(m * tamper_rate.get(ED25519, 0.0)))
        if k:
            sel = rng.choice(m, size=k, replace=False)
            for j, i in enumerate(sel):
                mode = j % 3
                if mode == 0:
                    bit = int(rng.integers(0, 256))
                    sigs[i, bit // 8] ^= np.uint8(1 << (bit % 8))
                    tam[i] = T_FLIP_R
                elif mode == 1:
                    raw = bytearray(raws[i] if raws[i] else b"\x00")
                    bit = int(rng.integers(0, len(raw) * 8))
                    raw[bit // 8] ^= 1 << (bit % 8)
                    msgs[i] = np.frombuffer(hashlib.sha256(bytes(raw)).digest(), np.uint8)
                    tam[i] = T_FLIP_MSG
                else:
                    S = int.from_bytes(sigs[i, 32:].tobytes(), "little") + ED_L
                    sigs[i, 32:] = np.frombuffer(S.to_bytes(32, "little"), np.uint8)
                    tam[i] = T_S_PLUS_L
        parts[ED25519] = (sigs, msgs, pks, np.zeros((m, 64), np.uint8), tam)

    if curves_order is None:
        curves_order = np.concatenate([np.full(n_by_curve.get(c, 0), c, np.uint8) for c in (SECP256K1, SECP256R1, ED25519)])
    n = len(curves_order)
    W = Workload(name, curves_order.astype(np.uint8), np.zeros((n, 64), np.uint8), np.zeros((n, 32), np.uint8),
                 np.zeros((n, 32), np.uint8), np.zeros((n, 64), np.uint8), np.zeros(n, np.uint8))
    for c, (sigs, msgs, pks, pubs, tam) in parts.items():
        pos = np.nonzero(W.curves == c)[0]
        assert len(pos) == len(sigs)
        W.sigs[pos], W.msgs[pos], W.pks[pos], W.expect_key[pos], W.tamper[pos] = sigs, msgs, pks, pubs, tam
    return W


def c4_order(n: int, seed: int, mix=(0.4, 0.3, 0.3), max_request: int = 4096):
    """Curve tag per item for the mixed workload: single-curve requests whose
    sizes are floor(exp(U(0, ln max_request))) (log-uniform in 1..max_request),
    in random order, each curve filled to its quota of the mix."""
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    quota = [int(round(n * mix[0])), int(round(n * mix[1]))]
    quota.append(n - quota[0] - quota[1])
    left = list(quota)
    tags, sizes = [], []
    while sum(left):
        w = np.array(left, dtype=np.float64)
        c = int(rng.choice(3, p=w / w.sum()))
        size = int(np.floor(np.exp(rng.uniform(0.0, np.log(max_request)))))
        size = max(1, min(size, left[c]))
        tags.append(np.full(size, c, np.uint8))
        sizes.append(size)
        left[c] -= size
    return np.concatenate(tags), np.array(sizes, np.int64)


def config(name: str, seed: int | None = None, ctx=None, n: int | None = None) -> Workload:
    """Workloads with the shapes of the benchmark configurations c1..c4."""
    if name == "c1":
        return make({SECP256K1: n or 1024}, seed or 1001, {}, ctx, name=name)
    if name == "c2":
        return make({ED25519: n or 65536}, seed or 2001, {ED25519: 0.03}, ctx, name=name)
    if name == "c3":
        return make({SECP256R1: n or 262144}, seed or 3001, {SECP256R1: 0.01}, ctx, name=name, ecdsa_modes=(T_NO_POINT,))
    if name == "c4":
        total = n or 1048576
        order, sizes = c4_order(total, seed or 4001)
        counts = {c: int((order == c).sum()) for c in (SECP256K1, SECP256R1, ED25519)}
        rate = {SECP256K1: 0.02, SECP256R1: 0.02, ED25519: 0.02}
        W = make(counts, seed or 4001, rate, ctx, name=name, curves_order=order)
        W.requests = sizes
        return W
    raise ValueError(name)


def expected_check(W: Workload, out: np.ndarray, status: np.ndarray) -> dict:
    """Check results against the outcomes the generator knows (no oracle).
    out: (n, 64) mixed records; ed25519 validity in byte 0."""
    from ._lib import ST_BAD_SCALAR, ST_MISMATCH, ST_NO_POINT, ST_OK

    ecdsa = W.curves != ED25519
    ed = ~ecdsa
    bad = np.zeros(W.n, bool)
    t = W.tamper
    ok_e = ecdsa & (t == T_NONE)
    bad |= ok_e & ((status != ST_OK) | (out != W.expect_key).any(axis=1))
    np_e = ecdsa & (t == T_NO_POINT)
    bad |= np_e & ((status != ST_NO_POINT) | (out != 0).any(axis=1))
    fm_e = ecdsa & (t == T_FLIP_MSG)
    bad |= fm_e & ((status != ST_OK) | (out == W.expect_key).all(axis=1))
    bad |= ed & (t == T_NONE) & ((status != ST_OK) | (out[:, 0] != 1))
    bad |= ed & ((t == T_FLIP_R) | (t == T_FLIP_MSG)) & ((status != ST_MISMATCH) | (out[:, 0] != 0))
    bad |= ed & (t == T_S_PLUS_L) & ((status != ST_BAD_SCALAR) | (out[:, 0] != 0))
    return {"items": int(W.n), "mismatches": int(bad.sum()), "first_bad": [int(i) for i in np.nonzero(bad)[0][:5]]}
