"""Build the oracle's C restatement (test infrastructure) with gcc:

    python oracle/build_oracle.py

Output: oracle/libsigops_oracle.so (git-ignored; rebuilt on the GPU machine).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc", "sigops_oracle.c")
LIB = os.path.join(HERE, "libsigops_oracle.so")
DEPS = [SRC, os.path.join(HERE, "csrc", "sha512_k.inc"), os.path.join(HERE, "csrc", "sha512_h.inc")]


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in DEPS):
        return LIB
    cc = os.environ.get("CC", "gcc")
    subprocess.run([cc, "-O2", "-std=c11", "-shared", "-fPIC", "-pthread", "-o", LIB + ".tmp", SRC], check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
