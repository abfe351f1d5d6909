"""polymps_gb300 — GB300 (sm_103a) implementation of PolyMPS's per-step particle path.

The product is ``_build/libmpsgpu.so`` (C ABI in include/mpsgpu.h); this package holds
its CUDA sources (``csrc/``), the C++ host driver (``host/``), the ctypes mirror of the
ABI (``abi``, ``mps``) and the synthetic case generator (``cases``).
"""
from . import abi, cases  # noqa: F401

__all__ = ["abi", "cases", "mps", "build"]
