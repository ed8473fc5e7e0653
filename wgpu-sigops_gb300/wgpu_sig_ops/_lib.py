"""ctypes binding of libsigops.so (include/sigops.h).

The shared library is the product; this module only declares its C ABI.  It
fails loudly (ImportError) when the library has not been built -- there is no
CPU fallback.
"""

from __future__ import annotations

import ctypes
import os

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("SIGOPS_LIB", os.path.join(_PKG_ROOT, "libsigops.so"))

SIGOPS_OK = 0
SIGOPS_E_INVAL = -22
SIGOPS_E_NOMEM = -12
SIGOPS_E_NODEV = -19
SIGOPS_E_CUDA = -5
SIGOPS_E_TABLE = -74
SIGOPS_E_TIMEDOUT = -110
SIGOPS_E_BUSY = -16
SIGOPS_E_RANGE = -34
SIGOPS_E_CANCELED = -125
SIGOPS_ALREADY_DONE = 1

SECP256K1, SECP256R1, ED25519 = 0, 1, 2

ST_OK, ST_BAD_SCALAR, ST_NO_POINT, ST_INFINITY, ST_MISMATCH = 0, 1, 2, 3, 4

_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t

# name -> (restype, argtypes); every function include/sigops.h declares
SIGNATURES = {
    "sigops_create": (_vp, [ctypes.c_int]),
    "sigops_destroy": (None, [_vp]),
    "sigops_last_error": (ctypes.c_char_p, []),
    "sigops_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "sigops_version": (ctypes.c_char_p, []),
    "sigops_bases_len": (ctypes.c_long, [ctypes.c_int, ctypes.c_uint32]),
    "sigops_bases": (ctypes.c_long, [ctypes.c_int, ctypes.c_uint32, _u32p, _sz]),
    "sigops_check_table": (ctypes.c_int, [ctypes.c_int, _u32p, _sz, ctypes.c_uint32]),
    "sigops_secp256k1_ecrecover": (ctypes.c_int, [_vp, _vp, _vp, _sz, _u32p, _sz, ctypes.c_uint32, _vp, _vp]),
    "sigops_secp256k1_ecrecover_single_shader": (ctypes.c_int, [_vp, _vp, _vp, _sz, ctypes.c_uint32, _vp, _vp]),
    "sigops_secp256r1_ecrecover": (ctypes.c_int, [_vp, _vp, _vp, _sz, _u32p, _sz, ctypes.c_uint32, _vp, _vp]),
    "sigops_secp256r1_ecrecover_single_shader": (ctypes.c_int, [_vp, _vp, _vp, _sz, ctypes.c_uint32, _vp, _vp]),
    "sigops_ed25519_ecverify": (ctypes.c_int, [_vp, _vp, _vp, _vp, _sz, _u32p, _sz, ctypes.c_uint32, _vp, _vp]),
    "sigops_ed25519_ecverify_single": (ctypes.c_int, [_vp, _vp, _vp, _vp, _sz, ctypes.c_uint32, _vp, _vp]),
    "sigops_ed25519_verify_raw": (ctypes.c_int, [_vp, _vp, _vp, _sz, _vp, _vp, _vp, _sz, _vp, _vp]),
    "sigops_plain_device": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, _sz, _vp, _vp, _vp]),
    "sigops_verify_mixed": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp]),
    "sigops_verify_mixed_device": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp, _vp]),
    "sigops_reserve": (ctypes.c_int, [_vp, _sz]),
    "sigops_verify_mixed_noalloc": (ctypes.c_int, [_vp, _vp, _vp, _vp, _sz, _vp, _vp, _vp]),
    "sigops_noalloc_status": (ctypes.c_int, [_vp]),
    "sigops_mixed_plan_create": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp, ctypes.POINTER(_vp)]),
    "sigops_mixed_plan_launch": (ctypes.c_int, [_vp, _vp]),
    "sigops_mixed_plan_destroy": (None, [_vp]),
    "sigops_set_variant": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "sigops_get_variant": (ctypes.c_int, [_vp, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 3),
    "sigops_autotune": (ctypes.c_int, [_vp, _sz, ctypes.c_char_p, _sz]),
    "sigops_workload_sign_ecdsa": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, _sz, _vp, _vp, _vp, _vp]),
    "sigops_workload_sign_ed25519": (ctypes.c_int, [_vp, _vp, _vp, _sz, _vp, _vp, _vp]),
    "sigops_server_create": (_vp, [_vp, ctypes.c_int, _sz, ctypes.c_double]),
    "sigops_server_destroy": (None, [_vp]),
    "sigops_server_slot_items": (_sz, [_vp]),
    "sigops_server_set_variant": (ctypes.c_int, [_vp, ctypes.c_int]),
    "sigops_server_set_adaptive": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_double]),
    "sigops_server_shape_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_double)]),
    "sigops_server_submit": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp, _vp, _vp, _sz, _vp, _vp, ctypes.POINTER(ctypes.c_uint64)]),
    "sigops_server_wait": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "sigops_server_cancel": (ctypes.c_int, [_vp, ctypes.c_uint64]),
    "sigops_server_dispatch_stats": (ctypes.c_int, [_vp, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "sigops_server_kernel_stats": (ctypes.c_int, [_vp, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "sigops_server_test_fault": (ctypes.c_int, [_vp, ctypes.c_int]),
    "sigops_test_fail_allocations": (ctypes.c_int, [ctypes.c_int]),
    "sigops_server_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                                           ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(_sz)]),
    "sigops_server_run_load": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_double)]),
    "sigops_sync": (ctypes.c_int, [_vp]),
    "sigops_probe_imad": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double)]),
    "sigops_probe_mul": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "sigops_probe_k1_lanes": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.c_size_t, _vp, _vp, ctypes.POINTER(ctypes.c_float)]),
    "sigops_probe_phase": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, ctypes.c_size_t, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_float)]),
    "sigops_test_wait_expiry": (ctypes.c_int, [_vp, ctypes.c_uint32]),
    "sigops_device_info": (ctypes.c_int, [_vp] + [ctypes.POINTER(ctypes.c_int)] * 4),
    "sigops_test_field": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _sz]),
    "sigops_test_sha512": (ctypes.c_int, [_vp, _vp, _vp, _sz]),
}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"libsigops.so not found at {LIB_PATH}; build it with "
            "`python wgpu-sigops_gb300/build_ext.py` (there is no CPU fallback)"
        )
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


class SigopsError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        msg = lib.sigops_last_error().decode(errors="replace")
        super().__init__(f"{where}: {lib.sigops_strerror(code).decode()} ({code}): {msg}")


def check(code: int, where: str) -> int:
    if code < 0:
        raise SigopsError(code, where)
    return code
