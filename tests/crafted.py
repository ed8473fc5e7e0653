"""ECDSA recovery inputs whose generator scalar u1 = -z / r (mod n) has chosen
16-bit windows, so that the signed window digits reach the ends of the
generator tables (+-32768, +-32767) in every window, for both 128-bit halves
of the GLV split as well.  Built from the oracle's curve arithmetic: pick a
nonce point R = k G with R.x < n, set r = R.x, choose u1 and u2, and solve
z = -u1 r, s = u2 r (mod n).  The expected key is whatever the oracle
recovers; the inputs only steer which table entries the kernels read."""
import random

from oracle import sigops_oracle as o


def _from_chunks(chunks):
    """16 little-endian 16-bit windows -> integer."""
    return sum((c & 0xFFFF) << (16 * j) for j, c in enumerate(chunks))


# window patterns (chunk j is bits 16j .. 16j+15)
PATTERNS = {
    # 0x7fff above a chunk whose top bit is set: digit +32768 (the last entry)
    "plus_max": [0xFFFF if j % 2 == 0 else 0x7FFF for j in range(16)],
    # 0x8000 above a chunk whose top bit is clear: digit -32768
    "minus_max": [0x0000 if j % 2 == 0 else 0x8000 for j in range(16)],
    # 0x8000 everywhere: -32768 in window 0, -32767 above it
    "all_8000": [0x8000] * 16,
    # 0x7fff everywhere: +32767 (the entry before the last)
    "all_7fff": [0x7FFF] * 16,
    # 0xffff everywhere but a clear top chunk: digits -1 with one carry at the top
    "ones": [0xFFFF] * 15 + [0x7FFF],
}


def crafted_signatures(c, seed=5):
    """[(name, sig64, msg32)] for curve c with u1 set to each pattern (and its
    negation), u2 random; s kept below 2^255 so that fuel's parity bit fits."""
    rng = random.Random(seed)
    out = []
    targets = []
    for name, chunks in PATTERNS.items():
        u1 = _from_chunks(chunks) % c.n
        targets += [(name, u1), ("neg_" + name, (-u1) % c.n)]
    for name, u1 in targets:
        while True:
            k = rng.randrange(1, c.n)
            R = o.ws_mul(c, k, c.g)
            if R[0] >= c.n:
                continue
            r = R[0]
            u2 = rng.randrange(1, c.n)
            s = u2 * r % c.n
            z = (-u1 * r) % c.n
            if s == 0 or s >= 2**255:
                continue
            sig = bytearray(r.to_bytes(32, "big") + s.to_bytes(32, "big"))
            sig[32] |= (R[1] & 1) << 7
            out.append((name, bytes(sig), z.to_bytes(32, "big")))
            break
    return out
