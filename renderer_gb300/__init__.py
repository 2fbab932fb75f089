"""renderer_gb300 — GB300-native unidirectional path-tracing hot path.

The compute path is the in-tree CUDA library renderer_gb300/_build/libgbrt.so
(built by renderer_gb300/build.py); this package only binds it. There is no
CPU fallback: loading fails loudly when the library is missing.
"""
import ctypes
import os

from . import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libgbrt.so")

_lib = None


class GbrtError(RuntimeError):
    def __init__(self, status, message):
        self.status = status
        super().__init__("%s: %s" % (_abi.STATUS_NAMES.get(status, status), message))


def lib():
    """The loaded C library (ctypes.CDLL) with every entry point typed."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libgbrt.so is not built (%s); run renderer_gb300/build.py or "
                              "__graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in _abi.SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, ctx=None):
    if status != _abi.OK:
        msg = lib().gbrt_last_error(ctx)
        raise GbrtError(status, msg.decode() if msg else "")


from .scene import SceneData  # noqa: E402
from .runtime import Context, GpuScene, PerPixelRenderer, UniDiPathTracingIntegrator  # noqa: E402

__all__ = ["lib", "check", "GbrtError", "SceneData", "Context", "GpuScene", "PerPixelRenderer",
           "UniDiPathTracingIntegrator"]
