"""Build helpers shared by the tests (compile on demand, in-tree)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "wgpu-sigops_gb300")
HOSTCHECK_SRC = os.path.join(ROOT, "tests", "hostcheck", "hostcheck.cpp")
HOSTCHECK_LIB = os.path.join(ROOT, "tests", "hostcheck", "libhostcheck.so")


def build_hostcheck() -> str:
    """g++ build of the kernels' arithmetic for the host (test-only library)."""
    deps = [HOSTCHECK_SRC] + [os.path.join(PKG, "csrc", f) for f in os.listdir(os.path.join(PKG, "csrc")) if f.endswith((".cuh", ".h"))]
    if os.path.exists(HOSTCHECK_LIB) and all(os.path.getmtime(HOSTCHECK_LIB) >= os.path.getmtime(d) for d in deps):
        return HOSTCHECK_LIB
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", HOSTCHECK_LIB + ".tmp", HOSTCHECK_SRC], check=True)
    os.replace(HOSTCHECK_LIB + ".tmp", HOSTCHECK_LIB)
    return HOSTCHECK_LIB


def build_lib() -> str:
    import sys

    sys.path.insert(0, PKG)
    import build_ext

    return build_ext.build()
