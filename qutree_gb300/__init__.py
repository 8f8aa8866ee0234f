"""GB300-native tree-tensor-network H.Psi sweep (QuTree's ML-MCTDH hot path).

Compute runs in libqtgpu.so (hand-written sm_103a CUDA behind the C ABI of
include/qtgpu.h); this package holds the ctypes binding (``qtgpu``), the
host-side model builders (``model``) and the build script (``build``).
"""
from . import model  # noqa: F401

__all__ = ["model", "qtgpu", "build"]
