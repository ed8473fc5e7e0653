"""wgpu_sig_ops on GB300: batch signature recovery / verification through
libsigops.so (hand-written sm_103a CUDA behind a C ABI).

Module layout mirrors the reference crate ``wgpu_sig_ops`` (src/lib.rs:1-10):
``secp256k1_ecdsa``, ``secp256r1_ecdsa``, ``ed25519_eddsa``, ``precompute``.
"""

from ._lib import SigopsError, lib  # noqa: F401  (loads the shared library)
from .context import Context, default_context  # noqa: F401


class ShaderFailureError(RuntimeError):
    """Raised when a batch call fails as a whole (src/lib.rs:12-14)."""


from . import batch, ed25519_eddsa, precompute, secp256k1_ecdsa, secp256r1_ecdsa  # noqa: E402,F401
