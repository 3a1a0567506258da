"""Writes tests/golden/converged.npz: converged images rendered by the CPU oracle.

The GPU's converged-image tests compare a high-spp GPU render (its own random streams)
against these images.  Each image is the mean of two independent oracle renders (seeds
1001 and 1002) of SPP / 2 passes each.  Their difference gives the noise still left in
the fixture, which is stored beside it:

    noise_<name> = mean(|a - b|^2) / 4 / mean(|(a + b) / 2|^2)

That is the relMSE of the stored image against the limit, estimated from the two halves.

Cases (64 x 64 unless stated; the scenes are gammaray_gb300.scenes functions):
  pt            displaced_sphere_lobes, path tracer, max depth 12, roulette after 10
  bdpt_mis_lt   displaced_sphere_lobes, BDPT with power-heuristic MIS and light tracing,
                path length 10, roulette from length 4
  bdpt_ref      cornell_spheres 48 x 48, BDPT with the reference's uniform weights
                (render/integrators.rs:343-418), path length 16, roulette from length 4

The BDPT with uniform weights on the displaced-sphere scene is not included.  Its
per-pixel error is heavy-tailed there: two independent 1024-spp renders differ by
relMSE 0.03-0.10, no less than at 256 spp.  The cause is connections between nearly
coincident vertices: their geometry term grows as 1/d^2, and uniform weights never
down-weight them.  A relMSE of 1e-3 is out of reach for that estimator at any feasible
spp.  The GPU tests check it per pixel at equal spp instead.

    python tests/golden/make_converged.py [spp]     # default 65536; 8 host threads take ~15 min
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import gammaray_gb300 as g  # noqa: E402
from gammaray_gb300 import _abi, scenes  # noqa: E402

SEEDS = (1001, 1002)


def cases():
    """(name, workload, integrator) of every converged image."""
    pt = scenes.displaced_sphere_lobes(64, 64)
    mis = scenes.displaced_sphere_lobes(64, 64, bdpt=True)
    cb = scenes.cornell_spheres(48, 48)
    return [
        ("pt", pt, pt.integrator),
        ("bdpt_mis_lt", mis, g.BdptIntegrator(max_depth=10, rr_depth=4, mis=1, light_tracing=1)),
        ("bdpt_ref", cb, g.BdptIntegrator()),
    ]


def render(lib, w, integ, spp, seed):
    st = g.Stage(w.prims, lib=lib, environment=w.environment, seed=seed)
    f = g.Film(w.width, w.height, lib=lib)
    st.render(w.camera, integ, f, spp)
    return f.resolve()


def main():
    spp = int(sys.argv[1]) if len(sys.argv) > 1 else 65536
    subprocess_make = os.path.join(ROOT, "oracle")
    os.system(f"make -s -C {subprocess_make}")
    lib = _abi.Lib(os.path.join(ROOT, "oracle", "libgammaray_ref.so"))
    out = {"spp": np.int64(spp), "seeds": np.asarray(SEEDS, np.int64)}
    for name, w, integ in cases():
        t0 = time.time()
        a = render(lib, w, integ, spp // 2, SEEDS[0])
        b = render(lib, w, integ, spp // 2, SEEDS[1])
        m = (0.5 * (a.astype(np.float64) + b)).astype(np.float32)
        noise = float(np.mean((a.astype(np.float64) - b) ** 2) / 4.0 / np.mean(m.astype(np.float64) ** 2))
        out[name] = m
        out["noise_" + name] = np.float64(noise)
        print(f"{name}: {w.width}x{w.height} {spp} spp, fixture noise relMSE {noise:.3e}, {time.time() - t0:.0f} s",
              flush=True)
    np.savez_compressed(os.path.join(HERE, "converged.npz"), **out)


if __name__ == "__main__":
    main()
