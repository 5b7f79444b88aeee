"""GB300-native explicit hot path of OpenRadioss.

The product is ``librg.so`` (CUDA kernels for sm_103a behind the C ABI of
``include/rg_api.h``).  This package holds its sources (``csrc/``), the
build recipe (``build.py``), the ctypes host mirror of the C ABI
(``engine.py``), host-side model preparation (``model.py``) and the batched
job server (``serving.py``).
"""
from . import model  # noqa: F401

__all__ = ["model", "engine", "build"]
