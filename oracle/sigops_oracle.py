"""CPU oracle for the batch signature path -- TEST INFRASTRUCTURE ONLY.

This module restates, in plain Python integers, what the reference crate
``wgpu_sig_ops`` (FuelLabs/wgpu-sigops) and the third-party crates it defers to
compute on the hot path:

* secp256k1 ECDSA public-key recovery with fuel-crypto's 64-byte signature
  encoding (fuel-crypto 0.49.0 -> secp256k1 0.26.0 / libsecp256k1),
* secp256r1 ECDSA public-key recovery (fuel-crypto -> p256 0.13.2 / ecdsa 0.16.9),
* ed25519 verification with ed25519-dalek 2.1.1 semantics (curve25519-dalek 4.1.3),
* the generator tables ``precompute::*_bases(log_limb_size)``.

It is the checker for the CUDA library, never part of it: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it.  Every function cites the reference file:line it follows (paths are
relative to the reference repository root).

Parity pins: ``tests/test_oracle.py`` checks this module against the golden
vectors in ``tests/golden/`` -- the reference's own secp256k1 known-answer test
(src/curve_algos/secp256k1_ecdsa.rs:206-214, 270-273, 285-289) and vectors
produced by independent implementations (OpenSSL through ``cryptography``,
libsodium through PyNaCl, ``hashlib``).  Behaviour on invalid inputs (r or s out
of range, r with no curve point, non-canonical S) follows the documented
behaviour of libsecp256k1 / p256 / dalek; the reference has no test for it.
"""

from __future__ import annotations

import hashlib
import hmac

# ---------------------------------------------------------------------------
# Per-item status codes (shared with include/sigops.h)
# ---------------------------------------------------------------------------
ST_OK = 0
ST_BAD_SCALAR = 1  # ECDSA: r or s outside [1, n-1]; ed25519: S >= l
ST_NO_POINT = 2    # ECDSA: r is not the x-coordinate of a point; ed25519: A does not decompress
ST_INFINITY = 3    # ECDSA: recovered key is the point at infinity
ST_MISMATCH = 4    # ed25519: [S]B - [k]A does not compress to R

# ---------------------------------------------------------------------------
# Curve constants (src/moduli.rs:1-50, src/tests/mod.rs:38-64)
# ---------------------------------------------------------------------------


class WeierstrassCurve:
    """Short Weierstrass curve y^2 = x^3 + a x + b over F_p with prime order n."""

    def __init__(self, name, p, n, a, b, gx, gy):
        self.name, self.p, self.n, self.a, self.b = name, p, n, a % p, b
        self.g = (gx, gy)


SECP256K1 = WeierstrassCurve(
    "secp256k1",
    p=2**256 - 2**32 - 977,
    n=0xFFFFFFFFFFFFFFFFFFFFFFFFFFFFFFFEBAAEDCE6AF48A03BBFD25E8CD0364141,
    a=0,
    b=7,  # src/tests/mod.rs:38-40
    gx=0x79BE667EF9DCBBAC55A06295CE870B07029BFCDB2DCE28D959F2815B16F81798,
    gy=0x483ADA7726A3C4655DA4FBFC0E1108A8FD17B448A68554199C47D08FFB10D4B8,
)

SECP256R1 = WeierstrassCurve(
    "secp256r1",
    p=2**256 - 2**224 + 2**192 + 2**96 - 1,
    n=0xFFFFFFFF00000000FFFFFFFFFFFFFFFFBCE6FAADA7179E84F3B9CAC2FC632551,
    a=-3,  # src/tests/mod.rs:42-48 (a = p - 3)
    b=0x5AC635D8AA3A93E7B3EBBD55769886BC651D06B0CC53B0F63BCE3C3E27D2604B,  # src/tests/mod.rs:50-56
    gx=0x6B17D1F2E12C4247F8BCE6E563A440F277037D812DEB33A0F4A13945D898C296,
    gy=0x4FE342E2FE1A7F9B8EE7EB4A7C0F9E162BCE33576B315ECECBB6406837BF51F5,
)

ED_P = 2**255 - 19
ED_L = 2**252 + 27742317777372353535851937790883648493
ED_D = (-121665 * pow(121666, -1, ED_P)) % ED_P
ED_SQRT_M1 = pow(2, (ED_P - 1) // 4, ED_P)
ED_BY = (4 * pow(5, -1, ED_P)) % ED_P


def _ed_recover_x(y: int, sign: int) -> int | None:
    xx = (y * y - 1) * pow(ED_D * y * y + 1, -1, ED_P) % ED_P
    x = pow(xx, (ED_P + 3) // 8, ED_P)
    if (x * x - xx) % ED_P != 0:
        x = x * ED_SQRT_M1 % ED_P
    if (x * x - xx) % ED_P != 0:
        return None
    if x & 1 != sign:
        x = ED_P - x
    return x


ED_BX = _ed_recover_x(ED_BY, 0)
ED_B = (ED_BX, ED_BY)

# ---------------------------------------------------------------------------
# Weierstrass arithmetic (Jacobian coordinates; None is the point at infinity)
# Plays the role of arkworks' Projective in src/curve_algos/secp256k1_ecdsa.rs:66-120
# ---------------------------------------------------------------------------


def _jac_double(c: WeierstrassCurve, P):
    if P is None:
        return None
    X, Y, Z = P
    p = c.p
    if Y == 0:
        return None
    YY = Y * Y % p
    S = 4 * X * YY % p
    ZZ = Z * Z % p
    M = (3 * X * X + c.a * ZZ * ZZ) % p
    X3 = (M * M - 2 * S) % p
    Y3 = (M * (S - X3) - 8 * YY * YY) % p
    Z3 = 2 * Y * Z % p
    return (X3, Y3, Z3)


def _jac_add(c: WeierstrassCurve, P, Q):
    if P is None:
        return Q
    if Q is None:
        return P
    p = c.p
    X1, Y1, Z1 = P
    X2, Y2, Z2 = Q
    Z1Z1 = Z1 * Z1 % p
    Z2Z2 = Z2 * Z2 % p
    U1 = X1 * Z2Z2 % p
    U2 = X2 * Z1Z1 % p
    S1 = Y1 * Z2 * Z2Z2 % p
    S2 = Y2 * Z1 * Z1Z1 % p
    H = (U2 - U1) % p
    R = (S2 - S1) % p
    if H == 0:
        if R == 0:
            return _jac_double(c, P)
        return None
    HH = H * H % p
    HHH = H * HH % p
    V = U1 * HH % p
    X3 = (R * R - HHH - 2 * V) % p
    Y3 = (R * (V - X3) - S1 * HHH) % p
    Z3 = Z1 * Z2 * H % p
    return (X3, Y3, Z3)


def _jac_neg(c, P):
    if P is None:
        return None
    return (P[0], (-P[1]) % c.p, P[2])


def _to_affine(c: WeierstrassCurve, P):
    if P is None:
        return None
    X, Y, Z = P
    zi = pow(Z, -1, c.p)
    zi2 = zi * zi % c.p
    return (X * zi2 % c.p, Y * zi2 * zi % c.p)


def ws_mul(c: WeierstrassCurve, k: int, A):
    """k * A for an affine point A (None = infinity); left-to-right double-and-add."""
    if A is None or k % c.n == 0:
        return None
    k %= c.n
    P = None
    Aj = (A[0], A[1], 1)
    for bit in bin(k)[2:]:
        P = _jac_double(c, P)
        if bit == "1":
            P = _jac_add(c, P, Aj)
    return _to_affine(c, P)


def ws_lincomb(c: WeierstrassCurve, k1: int, A, k2: int, B):
    """k1*A + k2*B (Shamir's trick), affine in, affine or None out."""
    k1 %= c.n
    k2 %= c.n
    Aj = None if A is None else (A[0], A[1], 1)
    Bj = None if B is None else (B[0], B[1], 1)
    ABj = _jac_add(c, Aj, Bj)
    P = None
    for i in range(max(k1.bit_length(), k2.bit_length()) - 1, -1, -1):
        P = _jac_double(c, P)
        b1, b2 = (k1 >> i) & 1, (k2 >> i) & 1
        if b1 and b2:
            P = _jac_add(c, P, ABj)
        elif b1:
            P = _jac_add(c, P, Aj)
        elif b2:
            P = _jac_add(c, P, Bj)
    return _to_affine(c, P)


def ws_on_curve(c: WeierstrassCurve, A) -> bool:
    x, y = A
    return (y * y - (x * x * x + c.a * x + c.b)) % c.p == 0


def ws_sqrt(c: WeierstrassCurve, v: int) -> int | None:
    """Square root for p = 3 mod 4 (src/wgsl/secp256k1_curve.wgsl:12-21), checked."""
    y = pow(v, (c.p + 1) // 4, c.p)
    if y * y % c.p != v % c.p:
        return None
    return y


# ---------------------------------------------------------------------------
# ECDSA recovery (fuel-crypto signature encoding)
# ---------------------------------------------------------------------------


def fuel_decode_signature(sig64: bytes) -> tuple[bytes, bool]:
    """Split off fuel's recovery bit (bit 7 of s[0]).

    src/tests/mod.rs:151-156 and src/wgsl/signature.wgsl:6-21.
    """
    sig = bytearray(sig64)
    is_y_odd = (sig[32] & 0x80) != 0
    sig[32] &= 0x7F
    return bytes(sig), is_y_odd


def ecdsa_recover(c: WeierstrassCurve, sig64: bytes, msg32: bytes) -> tuple[int, bytes]:
    """Recover the signer's key; returns (status, 64-byte x||y big-endian or b"").

    Follows ``arkworks_recover`` (src/curve_algos/secp256k1_ecdsa.rs:66-120,
    src/curve_algos/secp256r1_ecdsa.rs:63-117) and the one-kernel WGSL path
    (src/wgsl/secp256k1_ecdsa.wgsl:87-130), with the parse/validity rules of the
    crates the reference defers to (libsecp256k1 ``recover_ecdsa``, p256
    ``recover_from_prehash``):

    * r, s must lie in [1, n-1] (signature parse), else ST_BAD_SCALAR;
    * z = message mod n (scalar_set_b32 / Reduce::reduce_bytes);
    * R.x = r (fuel's one recovery bit carries only the y parity);
    * no square root of r^3 + a r + b -> ST_NO_POINT;
    * Q = r^-1 (s R - z G); Q at infinity -> ST_INFINITY.
    """
    if len(sig64) != 64 or len(msg32) != 32:
        raise ValueError("signature must be 64 bytes and message 32 bytes")
    sig, is_y_odd = fuel_decode_signature(sig64)
    r = int.from_bytes(sig[:32], "big")
    s = int.from_bytes(sig[32:], "big")
    n, p = c.n, c.p
    if not (1 <= r < n and 1 <= s < n):
        return ST_BAD_SCALAR, b""
    z = int.from_bytes(msg32, "big") % n
    x = r
    rhs = (x * x * x + c.a * x + c.b) % p
    y = ws_sqrt(c, rhs)
    if y is None:
        return ST_NO_POINT, b""
    if (y & 1) != int(is_y_odd):
        y = (p - y) % p
    rinv = pow(r, -1, n)
    u1 = (-z * rinv) % n
    u2 = (s * rinv) % n
    Q = ws_lincomb(c, u1, c.g, u2, (x, y))
    if Q is None:
        return ST_INFINITY, b""
    return ST_OK, Q[0].to_bytes(32, "big") + Q[1].to_bytes(32, "big")


def secp256k1_ecrecover(sig64: bytes, msg32: bytes) -> tuple[int, bytes]:
    """``secp256k1_ecdsa::ecrecover`` per item (src/secp256k1_ecdsa.rs:61-213)."""
    return ecdsa_recover(SECP256K1, sig64, msg32)


def secp256r1_ecrecover(sig64: bytes, msg32: bytes) -> tuple[int, bytes]:
    """``secp256r1_ecdsa::ecrecover`` per item (src/secp256r1_ecdsa.rs)."""
    return ecdsa_recover(SECP256R1, sig64, msg32)


# ---------------------------------------------------------------------------
# ed25519 (extended twisted Edwards, a = -1)
# ---------------------------------------------------------------------------


def _ed_add(P, Q):
    """add-2008-hwcd-3 (src/wgsl/ed25519_curve.wgsl:19-60), complete for ed25519."""
    p = ED_P
    X1, Y1, Z1, T1 = P
    X2, Y2, Z2, T2 = Q
    A = (Y1 - X1) * (Y2 - X2) % p
    B = (Y1 + X1) * (Y2 + X2) % p
    C = T1 * 2 * ED_D * T2 % p
    D = Z1 * 2 * Z2 % p
    E, F, G, H = B - A, D - C, D + C, B + A
    return (E * F % p, G * H % p, F * G % p, E * H % p)


ED_IDENTITY = (0, 1, 1, 0)


def _ed_ext(A):
    return (A[0], A[1], 1, A[0] * A[1] % ED_P)


def ed_mul(k: int, A):
    """k * A, affine in/out (double-and-add; src/wgsl/ed25519_curve.wgsl:106-135)."""
    P = ED_IDENTITY
    Aj = _ed_ext(A)
    for bit in bin(k)[2:] if k else "":
        P = _ed_add(P, P)
        if bit == "1":
            P = _ed_add(P, Aj)
    return ed_affine(P)


def ed_affine(P):
    X, Y, Z, _ = P
    zi = pow(Z, -1, ED_P)
    return (X * zi % ED_P, Y * zi % ED_P)


def ed_compress(A) -> bytes:
    """Canonical y little-endian, x parity in bit 255 (``compress_eteaffine``,
    src/wgsl/ed25519_curve.wgsl; curve25519-dalek ``EdwardsPoint::compress``)."""
    x, y = A
    b = bytearray(y.to_bytes(32, "little"))
    b[31] |= (x & 1) << 7
    return bytes(b)


def _sqrt_ratio_i(u: int, v: int) -> tuple[bool, int]:
    """curve25519-dalek ``FieldElement::sqrt_ratio_i``, as restated in
    src/curve_algos/ed25519_eddsa.rs:160-184 (and src/wgsl/ed25519_utils.wgsl:42-88)."""
    p = ED_P
    v3 = v * v * v % p
    v7 = v3 * v3 * v % p
    r = u * v3 * pow(u * v7, (p - 5) // 8, p) % p
    check = v * r * r % p
    correct = check == u % p
    flipped = check == (-u) % p
    flipped_i = check == (-u * ED_SQRT_M1) % p
    if flipped or flipped_i:
        r = r * ED_SQRT_M1 % p
    if r & 1:
        r = (p - r) % p
    return (correct or flipped), r


def ed_decompress(a32: bytes):
    """curve25519-dalek ``CompressedEdwardsY::decompress`` (dalek semantics).

    src/curve_algos/ed25519_eddsa.rs:79-103: y is read from the low 255 bits
    and taken mod p (a non-canonical y >= p is accepted); x is the non-negative
    root of (y^2-1)/(d y^2+1), negated when the sign bit is set (so x = 0 with
    the sign bit set is accepted).  Returns the affine point or None.
    """
    sign = a32[31] >> 7
    y = int.from_bytes(a32, "little") & ((1 << 255) - 1)
    y %= ED_P
    u = (y * y - 1) % ED_P
    v = (ED_D * y * y + 1) % ED_P
    ok, x = _sqrt_ratio_i(u, v)
    if not ok:
        return None
    if sign:
        x = (-x) % ED_P
    return (x, y)


def ed25519_ecverify(sig64: bytes, msg32: bytes, pk32: bytes) -> tuple[int, bool]:
    """ed25519-dalek 2.1.1 ``VerifyingKey::verify`` per item.

    Follows ``curve25519_ecverify`` (src/curve_algos/ed25519_eddsa.rs:49-77) and
    the one-kernel WGSL path (src/wgsl/main/ed25519_eddsa_main.wgsl:23-113):
    k = SHA-512(R || A || M) mod l and the check compress([S]B - [k]A) == R
    byte for byte.  Unlike the reference GPU path (which uses S raw,
    src/wgsl/main/ed25519_eddsa_main_0.wgsl:45-54) dalek built without
    ``legacy_compatibility`` (Cargo.toml:20) rejects S >= l.  The key A is
    decompressed first, as constructing a ``VerifyingKey`` does.
    """
    if len(sig64) != 64 or len(msg32) != 32 or len(pk32) != 32:
        raise ValueError("signature 64, message 32 and key 32 bytes expected")
    return ed25519_verify_raw(sig64, msg32, pk32)


def ed25519_verify_raw(sig64: bytes, msg: bytes, pk32: bytes) -> tuple[int, bool]:
    """The same check for a message of any length (ed25519-dalek
    ``VerifyingKey::verify(&[u8], &Signature)``); the reference's own API only
    passes 32-byte fuel messages (src/ed25519_eddsa.rs:67-74)."""
    if len(sig64) != 64 or len(pk32) != 32:
        raise ValueError("signature 64 and key 32 bytes expected")
    msg32 = bytes(msg)
    A = ed_decompress(pk32)
    if A is None:
        return ST_NO_POINT, False
    R_bytes = sig64[:32]
    S = int.from_bytes(sig64[32:], "little")
    if S >= ED_L:
        return ST_BAD_SCALAR, False
    k = int.from_bytes(hashlib.sha512(R_bytes + pk32 + msg32).digest(), "little") % ED_L
    minus_A = ((-A[0]) % ED_P, A[1])
    Rp = _ed_lincomb(S, ED_B, k, minus_A)
    if ed_compress(Rp) == R_bytes:
        return ST_OK, True
    return ST_MISMATCH, False


def _ed_lincomb(k1, A, k2, B):
    Aj, Bj = _ed_ext(A), _ed_ext(B)
    ABj = _ed_add(Aj, Bj)
    P = ED_IDENTITY
    for i in range(max(k1.bit_length(), k2.bit_length()) - 1, -1, -1):
        P = _ed_add(P, P)
        b1, b2 = (k1 >> i) & 1, (k2 >> i) & 1
        if b1 and b2:
            P = _ed_add(P, ABj)
        elif b1:
            P = _ed_add(P, Aj)
        elif b2:
            P = _ed_add(P, Bj)
    return ed_affine(P)


# ---------------------------------------------------------------------------
# Generator tables: precompute::*_bases(log_limb_size)  (src/precompute.rs:12-69)
# ---------------------------------------------------------------------------
WINDOW_SIZE = 4  # src/precompute.rs:12
MIN_LOG_LIMB_SIZE, MAX_LOG_LIMB_SIZE = 11, 15  # range the WGSL Montgomery path supports (src/wgsl/mont.wgsl:12,37)


def num_limbs(log_limb_size: int) -> int:
    """Limbs needed for 256 bits at ``log_limb_size`` bits per limb (multiprecision
    ``calc_num_limbs(log_limb_size, 256)``, src/shader.rs:51): ceil(256 / L) for
    every L the reference supports (11..15, none of which divides 256)."""
    return -(-256 // log_limb_size)


def to_limbs_le(v: int, log_limb_size: int) -> list[int]:
    """multiprecision ``bigint::from_biguint_le`` (src/tests/mod.rs:66-149)."""
    mask = (1 << log_limb_size) - 1
    return [(v >> (log_limb_size * i)) & mask for i in range(num_limbs(log_limb_size))]


def from_limbs_le(limbs, log_limb_size: int) -> int:
    return sum(int(l) << (log_limb_size * i) for i, l in enumerate(limbs))


def mont_radix(log_limb_size: int) -> int:
    """R = 2^(L * num_limbs) (multiprecision ``calc_mont_radix``, src/shader.rs:55)."""
    return 1 << (log_limb_size * num_limbs(log_limb_size))


def _check_log_limb_size(log_limb_size: int):
    if not (MIN_LOG_LIMB_SIZE <= log_limb_size <= MAX_LOG_LIMB_SIZE):
        raise ValueError(f"log_limb_size must be in [{MIN_LOG_LIMB_SIZE}, {MAX_LOG_LIMB_SIZE}]")


def ws_bases(c: WeierstrassCurve, log_limb_size: int) -> list[int]:
    """``secp256k1_bases`` / ``secp256r1_bases`` (src/precompute.rs:14-51):
    [1G .. 16G] affine (``precompute_table``, src/curve_algos/precompute.rs:1-17),
    each as x*R mod p then y*R mod p in L-bit little-endian limbs
    (``projectivexy_to_mont_limbs``, src/tests/mod.rs:134-149)."""
    _check_log_limb_size(log_limb_size)
    R = mont_radix(log_limb_size)
    out = []
    for i in range(1, (1 << WINDOW_SIZE) + 1):
        x, y = ws_mul(c, i, c.g)
        out += to_limbs_le(x * R % c.p, log_limb_size)
        out += to_limbs_le(y * R % c.p, log_limb_size)
    return out


def ed25519_bases(log_limb_size: int) -> list[int]:
    """``ed25519_bases`` (src/precompute.rs:54-69): [1B .. 16B] as x, y, t=x*y in
    Montgomery form (``eteprojective_to_xyt_mont_limbs``, src/tests/mod.rs:95-114)."""
    _check_log_limb_size(log_limb_size)
    R = mont_radix(log_limb_size)
    out = []
    for i in range(1, (1 << WINDOW_SIZE) + 1):
        x, y = ed_mul(i, ED_B)
        t = x * y % ED_P
        for v in (x, y, t):
            out += to_limbs_le(v * R % ED_P, log_limb_size)
    return out


def secp256k1_bases(log_limb_size: int) -> list[int]:
    return ws_bases(SECP256K1, log_limb_size)


def secp256r1_bases(log_limb_size: int) -> list[int]:
    return ws_bases(SECP256R1, log_limb_size)


# ---------------------------------------------------------------------------
# Signing helpers (for building test inputs; not on the verified path)
# ---------------------------------------------------------------------------


def fuel_message(data: bytes) -> bytes:
    """fuel-crypto ``Message::new(bytes)``: the SHA-256 digest of the bytes
    (used by src/tests/ed25519_eddsa.rs:17-20 and src/curve_algos/secp256k1_ecdsa.rs:160-161)."""
    return hashlib.sha256(data).digest()


def _rfc6979_nonce(secret: int, digest: bytes, n: int) -> int:
    """RFC 6979 section 3.2 deterministic nonce with HMAC-SHA256 (256-bit n)."""
    x = secret.to_bytes(32, "big")
    h = (int.from_bytes(digest, "big") % n).to_bytes(32, "big")
    V = b"\x01" * 32
    K = b"\x00" * 32
    K = hmac.new(K, V + b"\x00" + x + h, hashlib.sha256).digest()
    V = hmac.new(K, V, hashlib.sha256).digest()
    K = hmac.new(K, V + b"\x01" + x + h, hashlib.sha256).digest()
    V = hmac.new(K, V, hashlib.sha256).digest()
    while True:
        V = hmac.new(K, V, hashlib.sha256).digest()
        k = int.from_bytes(V, "big")
        if 1 <= k < n:
            return k
        K = hmac.new(K, V + b"\x00", hashlib.sha256).digest()
        V = hmac.new(K, V, hashlib.sha256).digest()


def ecdsa_sign_fuel(c: WeierstrassCurve, secret: int, digest32: bytes, k: int | None = None) -> bytes:
    """Low-s ECDSA signature over a 32-byte digest, recovery parity in bit 7 of
    s[0] (fuel-crypto ``Signature::sign`` / ``sign_prehashed`` encoding)."""
    n = c.n
    z = int.from_bytes(digest32, "big") % n
    while True:
        if k is None:
            k = _rfc6979_nonce(secret, digest32, n)
        R = ws_mul(c, k, c.g)
        r = R[0] % n
        if r != 0 and R[0] < n:
            s = pow(k, -1, n) * (z + r * secret) % n
            if s != 0:
                break
        k = (k + 1) % n or 1
    odd = R[1] & 1
    if s > n // 2:
        s = n - s
        odd ^= 1
    out = bytearray(r.to_bytes(32, "big") + s.to_bytes(32, "big"))
    out[32] |= odd << 7
    return bytes(out)


def ws_public_key(c: WeierstrassCurve, secret: int) -> bytes:
    x, y = ws_mul(c, secret, c.g)
    return x.to_bytes(32, "big") + y.to_bytes(32, "big")


def ed25519_keypair(seed32: bytes) -> tuple[int, bytes, bytes]:
    """RFC 8032 key expansion: (clamped scalar a, prefix, public key bytes)."""
    h = hashlib.sha512(seed32).digest()
    a = int.from_bytes(h[:32], "little")
    a &= (1 << 254) - 8
    a |= 1 << 254
    return a, h[32:], ed_compress(ed_mul(a, ED_B))


def ed25519_sign(seed32: bytes, msg: bytes) -> bytes:
    """RFC 8032 Ed25519 signing (what ed25519-dalek ``SigningKey::sign`` computes)."""
    a, prefix, A = ed25519_keypair(seed32)
    r = int.from_bytes(hashlib.sha512(prefix + msg).digest(), "little") % ED_L
    R = ed_compress(ed_mul(r, ED_B))
    k = int.from_bytes(hashlib.sha512(R + A + msg).digest(), "little") % ED_L
    S = (r + k * a) % ED_L
    return R + S.to_bytes(32, "little")
