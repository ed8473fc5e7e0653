"""Owning wrapper of a ``sigops_ctx`` (one CUDA stream + resident tables)."""

from __future__ import annotations

import ctypes
import threading

from ._lib import check, lib


class Context:
    def __init__(self, device: int = 0):
        self.ptr = lib.sigops_create(device)
        if not self.ptr:
            raise RuntimeError("sigops_create failed: " + lib.sigops_last_error().decode())
        self.device = device

    def close(self):
        if self.ptr:
            lib.sigops_destroy(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        check(lib.sigops_sync(self.ptr), "sigops_sync")

    def probe_imad(self) -> float:
        v = ctypes.c_double()
        check(lib.sigops_probe_imad(self.ptr, ctypes.byref(v)), "sigops_probe_imad")
        return v.value

    def probe_mul(self, form: int) -> float:
        """Multiply instructions per second of one form: 0 mad.lo, 1 mad.hi,
        2 mad.lo.cc/madc.hi.cc carry-chain rows, 3 mad.wide."""
        v = ctypes.c_double()
        check(lib.sigops_probe_mul(self.ptr, form, ctypes.byref(v)), "sigops_probe_mul")
        return v.value

    def autotune(self, probe_items: int = 0) -> dict:
        """Time every launch variant on a device-signed probe batch and keep the fastest."""
        import json

        buf = ctypes.create_string_buffer(16384)
        check(lib.sigops_autotune(self.ptr, probe_items, buf, len(buf)), "sigops_autotune")
        return json.loads(buf.value.decode())

    def set_variant(self, kernel: int, variant: int):
        """kernel 0..2: plain kernel of that curve; 3: the batched engine."""
        check(lib.sigops_set_variant(self.ptr, kernel, variant), "sigops_set_variant")

    def variants(self) -> dict:
        out = {}
        for k, name in enumerate(("plain_secp256k1", "plain_secp256r1", "plain_ed25519", "batched")):
            v, g, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            check(lib.sigops_get_variant(self.ptr, k, ctypes.byref(v), ctypes.byref(g), ctypes.byref(b)), "sigops_get_variant")
            out[name] = {"variant": v.value, "grid": g.value, "block": b.value}
        return out

    def device_info(self) -> dict:
        vals = [ctypes.c_int() for _ in range(4)]
        check(lib.sigops_device_info(self.ptr, *[ctypes.byref(v) for v in vals]), "sigops_device_info")
        return {"num_sms": vals[0].value, "plain_grid": [v.value for v in vals[1:]]}


_default = None
_default_lock = threading.Lock()


def default_context() -> Context:
    global _default
    with _default_lock:
        if _default is None:
            _default = Context(0)
        return _default
