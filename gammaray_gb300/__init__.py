"""gammaray_gb300 — the rendering hot path of sdao/gammaray on GB300 (sm_103a).

The product is `libgammaray_gpu.so` (hand-written CUDA, C ABI in include/gammaray.h),
built in-tree by `gammaray_gb300.build.build()`.  This package is the host side over
that ABI: a mirror of the reference's Rust API (`api`), the seeded benchmark scenes
(`scenes`) and the batching / serving drivers.  There is no CPU fallback: `load()`
raises when the CUDA library is missing.
"""
from __future__ import annotations

import os

from . import _abi

PACKAGE_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PACKAGE_DIR, "libgammaray_gpu.so")

_lib = None


def load() -> _abi.Lib:
    """The CUDA library (loaded once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the CUDA library has no CPU fallback)")
        _lib = _abi.Lib(LIB_PATH)
        if _lib.backend != "cuda-sm_103a":
            raise RuntimeError(f"{LIB_PATH} reports backend {_lib.backend!r}, expected the CUDA library")
    return _lib


from .api import (  # noqa: E402
    BdptIntegrator,
    Camera,
    DisplayColorIntegrator,
    Film,
    Mat,
    Material,
    Mesh,
    PathTracerIntegrator,
    Quat,
    Sphere,
    Stage,
    bsdf_eval,
    bsdf_pdf,
    bsdf_sample,
    light_eval,
)

__all__ = [
    "load", "Camera", "Film", "Mat", "Material", "Mesh", "PathTracerIntegrator", "BdptIntegrator",
    "DisplayColorIntegrator", "Quat", "Sphere", "Stage", "bsdf_eval", "bsdf_pdf", "bsdf_sample", "light_eval",
]
