"""Generate ed25519_raw.json: ed25519 signatures over messages of any length
(run in a container that has ``cryptography`` and ``PyNaCl``; the GPU test
machines only read the JSON).

    python tests/golden/make_golden_raw.py

Signatures come from OpenSSL (through ``cryptography``, RFC 8032 deterministic
signing, as ed25519-dalek).  Every vector's verdict is agreed by OpenSSL and by
libsodium (through PyNaCl); the generator asserts the agreement.  Message
lengths straddle the SHA-512 block boundaries of the challenge preimage
R || A || M (64 + len + 17 bytes of padded input: one block up to len = 47,
two up to 175, ...).  Cases: valid, flipped message byte, flipped R bit,
S + l (non-canonical S), and a signature checked against another key.
"""

from __future__ import annotations

import json
import os
import random

from cryptography.exceptions import InvalidSignature
from cryptography.hazmat.primitives import serialization
from cryptography.hazmat.primitives.asymmetric import ed25519
import nacl.exceptions
import nacl.signing

HERE = os.path.dirname(os.path.abspath(__file__))
L = 2**252 + 27742317777372353535851937790883648493
LENGTHS = [0, 1, 2, 31, 32, 33, 46, 47, 48, 49, 63, 64, 65, 110, 111, 112, 113, 127, 128, 129, 174, 175, 176, 177,
           239, 240, 255, 256, 300, 302, 303, 304, 500, 1000, 1023, 2047, 4096]


def openssl_ok(pk: bytes, sig: bytes, msg: bytes) -> bool:
    try:
        ed25519.Ed25519PublicKey.from_public_bytes(pk).verify(sig, msg)
        return True
    except (InvalidSignature, ValueError):
        return False


def sodium_ok(pk: bytes, sig: bytes, msg: bytes) -> bool:
    try:
        nacl.signing.VerifyKey(pk).verify(msg, sig)
        return True
    except (nacl.exceptions.BadSignatureError, nacl.exceptions.ValueError, ValueError):
        return False


def main():
    rng = random.Random(20240611)
    out = []
    for i, n in enumerate(LENGTHS):
        sk = ed25519.Ed25519PrivateKey.from_private_bytes(rng.randbytes(32))
        pk = sk.public_key().public_bytes(serialization.Encoding.Raw, serialization.PublicFormat.Raw)
        msg = rng.randbytes(n)
        sig = sk.sign(msg)
        cases = [("valid", sig, msg, pk)]
        if n:
            j = rng.randrange(n)
            cases.append(("flip_msg", sig, msg[:j] + bytes([msg[j] ^ 0x01]) + msg[j + 1:], pk))
        cases.append(("flip_r", bytes([sig[0] ^ 0x04]) + sig[1:], msg, pk))
        s_plus_l = (int.from_bytes(sig[32:], "little") + L).to_bytes(32, "little")
        cases.append(("s_plus_l", sig[:32] + s_plus_l, msg, pk))
        other = ed25519.Ed25519PrivateKey.from_private_bytes(rng.randbytes(32)).public_key()
        cases.append(("other_key", sig, msg, other.public_bytes(serialization.Encoding.Raw, serialization.PublicFormat.Raw)))
        for name, sg, m, k in cases:
            a, b = openssl_ok(k, sg, m), sodium_ok(k, sg, m)
            assert a == b, (name, n)
            out.append({"case": name, "len": n, "msg": m.hex(), "sig": sg.hex(), "pubkey": k.hex(), "valid": a})
    with open(os.path.join(HERE, "ed25519_raw.json"), "w") as f:
        json.dump({"ed25519_raw": out}, f, indent=0)
        f.write("\n")
    print(len(out), "vectors;", sum(v["valid"] for v in out), "valid")


if __name__ == "__main__":
    main()
