"""Writes the golden vectors of tests/golden/oracle_golden.npz from the CPU oracle.

The reference (Rust) has no tests or fixtures and cannot be built here, so these vectors
pin the oracle to itself over time and give the GPU tests fixed expected values:
closest hits of seeded rays (Cornell box with spheres; 102,422-triangle displaced
sphere), BSDF values and pdfs of seeded queries, a display-colour film (its weights
depend on the jitter only, its colours on the hit materials), and the SAH tree hashes.

    python tests/golden/make_golden.py          # rewrites the file
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import gammaray_gb300 as g  # noqa: E402
from gammaray_gb300 import _abi, scenes  # noqa: E402


def rays(n, seed, lo, hi, target=None):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3)) if target is None else rng.normal(size=(n, 3)) * 0.6 + (np.asarray(target) - o)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], axis=1).astype(np.float32)


def frames(n, rng):
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    t = np.cross(nrm, rng.normal(size=(n, 3)))
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    fr = np.zeros(n, _abi.FRAME_DTYPE)
    fr["normal"], fr["tangent"], fr["binormal"], fr["geom_normal"] = nrm, t, np.cross(nrm, t), nrm
    return fr


MATERIALS = {
    "default": lambda: g.Material.disney().build(),
    "metal": lambda: g.Material.disney().base_color((0.9, 0.6, 0.2)).metallic(1.0).roughness(0.2).build(),
    "glass": lambda: g.Material.disney().specular_trans(1.0).roughness(0.3).ior(1.5).build(),
}


def compute(lib, given=None):
    """The golden arrays computed by `lib`.  With `given` (a loaded file), the stored rays
    and BSDF queries are reused instead of drawn again, so a numpy whose random streams
    differ still checks the same inputs."""
    out = {}
    cornell = scenes.cornell_spheres(16, 16, 1)
    disp = scenes.displaced_sphere(16, 16, 1)
    sc = g.Stage(cornell.prims, lib=lib)
    sd = g.Stage(disp.prims, lib=lib)
    out["cornell_rays"] = rays(1024, 101, -0.9, 1.9) if given is None else given["cornell_rays"]
    out["cornell_hits"] = sc.intersect(out["cornell_rays"])
    out["disp_rays"] = (rays(1024, 102, -3.0, 3.0, target=(0, 0, 0)) if given is None
                        else given["disp_rays"])
    out["disp_hits"] = sd.intersect(out["disp_rays"])
    rng = np.random.default_rng(103)
    n = 256
    fr = frames(n, rng)
    wi = rng.normal(size=(n, 3))
    wi = (wi / np.linalg.norm(wi, axis=1, keepdims=True)).astype(np.float32)
    wo = rng.normal(size=(n, 3))
    wo = (wo / np.linalg.norm(wo, axis=1, keepdims=True)).astype(np.float32)
    if given is not None:
        fr, wi, wo = given["bsdf_frames"], given["bsdf_wi"], given["bsdf_wo"]
    out["bsdf_frames"], out["bsdf_wi"], out["bsdf_wo"] = fr, wi, wo
    for name, mk in MATERIALS.items():
        m = mk()
        out[f"bsdf_f_{name}"] = g.bsdf_eval(m, fr, wi, wo, True, lib=lib)
        out[f"bsdf_pdf_{name}"] = g.bsdf_pdf(m, fr, wi, wo, lib=lib)
    st = g.Stage(cornell.prims, lib=lib, seed=7)
    f = g.Film(24, 24, lib=lib)
    st.render(cornell.camera, g.DisplayColorIntegrator(), f, 3)
    out["display_accum"], out["display_weight"] = f.read()
    out["tree_hash"] = np.array([g.api.plan_scene(cornell.prims, lib=lib).tree_hash,
                                 g.api.plan_scene(disp.prims, lib=lib).tree_hash], np.uint64)
    return out


if __name__ == "__main__":
    oracle = _abi.Lib(os.path.join(ROOT, "oracle", "libgammaray_ref.so"))
    data = compute(oracle)
    path = os.path.join(HERE, "oracle_golden.npz")
    np.savez_compressed(path, **data)
    print(path, os.path.getsize(path), "bytes")
