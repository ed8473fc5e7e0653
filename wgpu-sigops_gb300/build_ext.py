"""Build libsigops.so in-tree (sm_103a only).

    python wgpu-sigops_gb300/build_ext.py [--force] [--jobs N]

Each translation unit compiles to ``_build/<name>.o`` in parallel, then nvcc
links the shared library next to this file.  Objects are reused when their
source tree hash and flags are unchanged.  No cmake.
"""

from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsigops.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["k_k1.cu", "k_r1.cu", "k_ed.cu", "k_sign.cu", "k_batched.cu", "k_batched_0.cu", "k_batched_1.cu", "k_batched_2.cu", "k_batched_3.cu", "k_batched_k1.cu", "k_batched_r1.cu", "k_batched_ed.cu", "k_batched_k1_w.cu", "k_batched_r1_w.cu", "k_batched_ed_w.cu", "k_misc.cu", "k_split.cu", "host.cu", "serving.cu", "noalloc.cu", "autotune.cu"]
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I" + INCLUDE, "-Xptxas", "-v"]


def _tree_hash() -> str:
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for name in sorted(os.listdir(d)):
            if name.endswith((".cu", ".cuh", ".h")):
                with open(os.path.join(d, name), "rb") as f:
                    h.update(name.encode() + b"\0" + f.read())
    h.update(" ".join(FLAGS).encode())
    return h.hexdigest()[:16]


def _compile(src: str, stamp: str) -> tuple[str, str]:
    obj = os.path.join(BUILD, src.replace(".cu", f".{stamp}.o"))
    log = os.path.join(BUILD, src.replace(".cu", ".ptxas.txt"))
    if os.path.exists(obj):
        return obj, ""
    cmd = [NVCC, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj + ".tmp"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    with open(log, "w") as f:
        f.write(" ".join(cmd) + "\n" + p.stdout + p.stderr)
    if p.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{p.stdout}\n{p.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj, p.stderr


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    """Compile (if needed) and return the path of libsigops.so."""
    os.makedirs(BUILD, exist_ok=True)
    stamp = _tree_hash()
    stamp_file = os.path.join(BUILD, "lib.stamp")
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file):
        with open(stamp_file) as f:
            if f.read().strip() == stamp:
                return LIB
    if force:
        for name in os.listdir(BUILD):
            if name.endswith(".o"):
                os.remove(os.path.join(BUILD, name))
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, stamp), SOURCES))
    if verbose:
        for _, err in results:
            if err:
                print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    cmd = [NVCC, *ARCH, "-shared", "-o", LIB + ".tmp", *objs]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stdout}\n{p.stderr}")
    os.replace(LIB + ".tmp", LIB)
    with open(stamp_file, "w") as f:
        f.write(stamp)
    # drop objects of older source trees
    for name in os.listdir(BUILD):
        if name.endswith(".o") and f".{stamp}." not in name:
            os.remove(os.path.join(BUILD, name))
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(a.force, a.jobs, a.verbose))
