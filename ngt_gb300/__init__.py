"""GB300-native batched k-NN search for NGT indexes.

The compute path is the native library libngtgpu.so (hand-written CUDA for
sm_103a behind NGT's C ABI); this package only loads it and offers a thin
Python mirror of NGT's ctypes wrapper (``ngt.base.Index``).
"""
from .base import build_onng, Index, ObjectDistance, NativeError, QBGIndex, QBGServer, QGServer, QuantizedIndex, Server, load_library  # noqa: F401


__all__ = ["build_onng", "Index", "ObjectDistance", "NativeError", "QBGIndex", "QBGServer", "QGServer", "QuantizedIndex", "Server", "load_library"]
