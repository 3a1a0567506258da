"""Images of the CUDA library against the oracle, with independent random streams.

Two checks, on the 102,400-triangle displaced-sphere scene (the path tracer's and the
BDPT's workload) with a metal and a sheen + clearcoat sphere added, so that every Disney
lobe is on screen (gammaray_gb300.scenes.displaced_sphere_lobes):

1. Converged image.  A 65536-spp GPU render is compared with the oracle's converged
   render of the same scene, committed as tests/golden/converged.npz with the script
   that makes it (tests/golden/make_converged.py).  The bar is relMSE <= 1e-3.
   4096 spp is not converged on this scene.  Measured with the oracle against itself,
   one 4096-spp render has a relMSE of about 1.2e-3 against the limit: caustics through
   the rough glass sphere, and highlights of the light in the clearcoats.  So the GPU
   renders 65536 spp, and the fixture is 65536 spp too.  Its own remaining noise is
   stored beside it and is printed.
   The BDPT with the reference's uniform weights is checked this way on the Cornell box.
   On the displaced sphere its error is heavy-tailed (see make_converged.py), so there it
   gets the per-pixel check only.
2. Per-pixel means at equal spp.  Each side renders K images from K seeds of its own, and
   the per-pixel Welch statistics must look like N(0, 1) (tests/pixelstats.py).
"""
from __future__ import annotations

import importlib.util
import os

import numpy as np
import pytest

import gammaray_gb300 as g
from gammaray_gb300 import scenes

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REL_MSE_BAR = 1e-3
GPU_SPP = 65536


def _cases():
    spec = importlib.util.spec_from_file_location("make_converged", os.path.join(HERE, "golden", "make_converged.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return {name: (w, integ) for name, w, integ in mod.cases()}


def _render(lib, w, integ, spp, seed):
    st = g.Stage(w.prims, lib=lib, environment=w.environment, seed=seed)
    f = g.Film(w.width, w.height, lib=lib)
    st.render(w.camera, integ, f, spp)
    return f.resolve()


@pytest.mark.parametrize("name", ["pt", "bdpt_mis_lt", "bdpt_ref"])
def test_converged_image_within_rel_mse(gpu, name):
    fix = np.load(os.path.join(HERE, "golden", "converged.npz"))
    w, integ = _cases()[name]
    ref = fix[name].astype(np.float64)
    img = _render(gpu, w, integ, GPU_SPP, seed=77).astype(np.float64)  # streams unlike the fixture's
    rel = float(np.mean((img - ref) ** 2) / np.mean(ref ** 2))
    print(f"{name}: relMSE {rel:.3e} against the {int(fix['spp'])}-spp oracle image "
          f"(its own noise {float(fix['noise_' + name]):.1e})")
    assert np.isfinite(img).all()
    assert rel <= REL_MSE_BAR, rel


@pytest.mark.parametrize("name", ["pt", "bdpt_mis_lt", "bdpt_ref"])
def test_pixel_means_agree_at_equal_spp(gpu, oracle, name):
    pytest.importorskip("scipy")
    from pixelstats import check_consistent

    bdpt = name != "pt"
    w = scenes.displaced_sphere_lobes(64, 64, bdpt=bdpt)
    integ = {"pt": w.integrator, "bdpt_mis_lt": g.BdptIntegrator(max_depth=10, rr_depth=4, mis=1, light_tracing=1),
             "bdpt_ref": g.BdptIntegrator(max_depth=10, rr_depth=4)}[name]
    K, n = 16, (32 if bdpt else 64)
    a = np.stack([_render(gpu, w, integ, n, 100 + k) for k in range(K)])
    b = np.stack([_render(oracle, w, integ, n, 500 + k) for k in range(K)])
    print(name, check_consistent(a, b))
