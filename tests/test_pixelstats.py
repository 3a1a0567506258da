"""The per-pixel check of tests/pixelstats.py, on the CPU oracle alone.

It passes for two sets of independent oracle renders (the same estimator, different
random streams).  It fails when one side carries a bias, planted here by scaling the
oracle's images on the CPU: 10% over the whole image (caught by the whole-image
deviate), or 25% on one 8 x 8-pixel block (caught by the block deviates).  These are
24 x 24 images at 16 x 64 spp; the GPU tests use 64 x 64 images, whose whole-image
deviate resolves smaller biases.
"""
from __future__ import annotations

import numpy as np
import pytest

import gammaray_gb300 as g
from gammaray_gb300 import scenes


def _renders(oracle, seeds, n):
    w = scenes.cornell_spheres(24, 24, 1)
    out = []
    for s in seeds:
        st = g.Stage(w.prims, lib=oracle, seed=s)
        f = g.Film(24, 24, lib=oracle)
        st.render(w.camera, w.integrator, f, n)
        out.append(f.resolve())
    return np.stack(out)


def test_pixel_check_passes_same_estimator_and_catches_a_bias(oracle):
    pytest.importorskip("scipy")
    from pixelstats import check_consistent

    a = _renders(oracle, range(100, 116), 64)
    b = _renders(oracle, range(500, 516), 64)
    check_consistent(a, b)
    with pytest.raises(AssertionError):
        check_consistent(a, b * np.float32(1.10))
    local = b.copy()
    local[:, 8:16, 8:16] *= np.float32(1.25)
    with pytest.raises(AssertionError):
        check_consistent(a, local)
