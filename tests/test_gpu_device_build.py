"""The device BVH build (GR_BUILD_DEVICE_LBVH) on the GPU: a different tree, the same
closest hits (ties at exactly equal distance aside), renders that match the host-built
scene's, and the degenerate inputs a linear BVH meets (one primitive, coincident
centroids, spheres only, attribute indices that must follow the primitives)."""
from __future__ import annotations

import numpy as np
import pytest

import gammaray_gb300 as g
from gammaray_gb300 import scenes
from test_gpu_parity import check_hits, random_rays

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("width,leaf", [(4, 2), (2, 1), (8, 4)])
def test_device_build_hits_equal_oracle(gpu, oracle, width, leaf):
    w = scenes.displaced_sphere(64, 64, 1)
    sd = g.Stage(w.prims, lib=gpu, bvh_width=width, leaf_size=leaf, device_build=True)
    so = g.Stage(w.prims, lib=oracle)
    rays = random_rays(1 << 20, 31 + width, target=(0, 0, 0))
    hits, ties, exact = check_hits(sd.intersect(rays), so.intersect(rays))
    assert hits > (1 << 19)
    assert exact == 1.0
    info = sd.info()
    assert info.num_wide_nodes > 0 and info.num_components == 102_422


def test_device_build_matches_naive_on_spheres_and_cornell(gpu):
    w = scenes.cornell_spheres()
    sd = g.Stage(w.prims, lib=gpu, device_build=True)
    rays = random_rays(1 << 16, 41, lo=-0.9, hi=1.9)
    check_hits(sd.intersect(rays), sd.intersect_naive(rays))
    spheres = [g.Sphere(g.Material.disney().build(), g.Mat.translation(tuple(c)), 0.2)
               for c in np.random.default_rng(5).uniform(-2, 2, (300, 3))]
    ss = g.Stage(spheres, lib=gpu, device_build=True)
    rays = random_rays(1 << 16, 42)
    check_hits(ss.intersect(rays), ss.intersect_naive(rays))


def test_device_build_degenerate_inputs(gpu):
    mat = g.Material.disney().build()
    one = g.Stage([g.Sphere(mat, None, 1.0)], lib=gpu, device_build=True)
    rays = random_rays(4096, 43)
    check_hits(one.intersect(rays), one.intersect_naive(rays))
    # 2,000 copies of one triangle: every Morton code equal, ties everywhere
    v = np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0]], np.float32)
    t = np.tile(np.array([[0, 1, 2]], np.uint32), (2000, 1))
    dup = g.Stage([g.Mesh(mat, None, v, t)], lib=gpu, device_build=True, leaf_size=2)
    rays = random_rays(4096, 44, target=(0, 0, 0))
    hd, hn = dup.intersect(rays), dup.intersect_naive(rays)
    assert ((hd["prim"] >= 0) == (hn["prim"] >= 0)).all()
    hit = hd["prim"] >= 0
    assert hit.any()
    np.testing.assert_array_equal(hd["t"][hit], hn["t"][hit])


def test_device_build_render_matches_host_build(gpu):
    # Shading normals and uvs follow their triangles into leaf order.
    w = scenes.displaced_sphere(64, 64, 4, tris=20_000)
    prims = list(w.prims)
    m = prims[0]
    n = np.random.default_rng(6).normal(size=(len(m.vertices), 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    prims[0] = g.Mesh(m.material, None, m.vertices, m.triangles, normals=n, tri_normals=m.triangles,
                      uvs=np.zeros((len(m.vertices), 2), np.float32), tri_uvs=m.triangles)
    films = []
    for dev in (False, True):
        st = g.Stage(prims, lib=gpu, environment=w.environment, seed=8, device_build=dev)
        f = g.Film(64, 64, lib=gpu)
        st.render(w.camera, w.integrator, f, 4)
        films.append(f.resolve())
    a, b = films
    rel = float(np.mean((a - b) ** 2) / np.mean(b ** 2))
    assert rel < 1e-6, rel


def test_device_build_time_and_bytes(gpu):
    w = scenes.displaced_sphere(64, 64, 1)
    g.Stage(scenes.cornell_spheres().prims, lib=gpu, device_build=True).close()  # kernels loaded
    host = g.Stage(w.prims, lib=gpu)
    dev = g.Stage(w.prims, lib=gpu, device_build=True)
    hi, di = host.info(), dev.info()
    assert di.device_bytes > 0 and di.num_wide_nodes <= di.num_components
    assert di.build_seconds < hi.build_seconds, (di.build_seconds, hi.build_seconds)
