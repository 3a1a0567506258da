"""Host-side logic without a GPU: the Python mirror of the reference API, the seeded
scenes, the product's host BVH build (gr_scene_plan, no device needed) against the
oracle's, and the replica bookkeeping on 2 gloo ranks."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

import gammaray_gb300 as g
from gammaray_gb300 import _abi, scenes


def test_disney_builder_defaults(oracle):
    import ctypes as C

    d = _abi.MaterialDesc()
    oracle.gr_material_disney_defaults(C.byref(d))
    assert bytes(g.Material.disney().build().desc) == bytes(d)
    m = g.Material.disney().base_color((0.1, 0.2, 0.3)).roughness(0.7).metallic(1).build()
    assert list(m.desc.base_color) == pytest.approx([0.1, 0.2, 0.3])
    assert m.desc.roughness == pytest.approx(0.7) and m.desc.metallic == 1.0


def test_camera_fov():
    c = g.Camera.with_fov(40.0)
    assert c.vertical_aperture / (2 * c.focal_length) == pytest.approx(np.tan(np.radians(20)))


def test_scene_sizes():
    w = scenes.displaced_sphere(64, 64, 1)
    assert w.num_triangles() == 102_400 + 20 + 2
    c = scenes.cornell_spheres()
    assert c.num_triangles() == 12 and sum(isinstance(p, g.Sphere) for p in c.prims) == 2
    a = scenes.displaced_sphere(64, 64, 1)
    assert np.array_equal(a.prims[0].vertices, w.prims[0].vertices)  # seeded: reproducible


def test_batch_and_serving_scene_ranges():
    b = scenes.batch_scenes(8)
    for w in b:
        assert 1_000 * 0.9 <= w.meta["triangles"] <= 200_000 * 1.1
        assert (w.width, w.height) in {(128, 128), (256, 256), (512, 512), (1024, 576)}
        assert 4 <= w.spp <= 64 and 4 <= w.integrator.max_depth <= 12


def gpu_lib():
    import gammaray_gb300

    if not os.path.exists(gammaray_gb300.LIB_PATH):
        try:
            from gammaray_gb300 import build

            build.build()
        except Exception as e:
            pytest.skip(f"cannot build the CUDA library here: {e}")
    return _abi.Lib(gammaray_gb300.LIB_PATH)


def test_product_host_build_matches_oracle_tree(oracle):
    # Both sides restate the reference SAH build; the binary trees must have the same
    # number of nodes, including the multi-component leaves of coincident centroids.
    lib = gpu_lib()
    for w in (scenes.displaced_sphere(8, 8, 1, tris=20_000), scenes.cornell_spheres()):
        a = g.api.plan_scene(w.prims, lib=lib)
        b = g.api.plan_scene(w.prims, lib=oracle)
        assert a.num_components == b.num_components
        assert a.num_binary_nodes == b.num_binary_nodes
        assert a.num_lights == b.num_lights


def test_threaded_host_build_is_the_reference_tree(oracle):
    # The product's build runs subtrees and large passes on threads; its binary tree
    # must be the serial restatement's exactly (boxes, leaf order, ids), at sizes that
    # use the threads (>= 32,768 components split their passes) and on skewed inputs.
    lib = gpu_lib()
    mat = g.Material.disney().build()
    rng = np.random.default_rng(9)
    verts = (rng.standard_cauchy(size=(60_000, 3)) * 0.1).astype(np.float32)  # heavy tails: skewed splits
    cases = [scenes.displaced_sphere(8, 8, 1, tris=120_000).prims,
             [g.Mesh(mat, None, verts, rng.integers(0, 60_000, (80_000, 3)).astype(np.uint32))],
             scenes.cornell_spheres().prims]
    for prims in cases:
        a = g.api.plan_scene(prims, lib=lib)
        b = g.api.plan_scene(prims, lib=oracle)
        assert a.num_binary_nodes == b.num_binary_nodes
        assert a.tree_hash == b.tree_hash != 0


def test_concurrent_host_builds_share_the_pass_pool(oracle):
    # Two host threads building at once (ctypes releases the GIL) share the library's
    # pass pool; each tree must still be the serial restatement's.
    import threading

    lib = gpu_lib()
    scenes_ = [scenes.displaced_sphere(8, 8, 1, tris=90_000).prims, scenes.displaced_sphere(8, 8, 1, tris=60_000).prims]
    want = [g.api.plan_scene(p, lib=oracle).tree_hash for p in scenes_]
    got = [[], []]

    def worker(k):
        for _ in range(3):
            got[k].append(g.api.plan_scene(scenes_[k], lib=lib).tree_hash)

    th = [threading.Thread(target=worker, args=(k,)) for k in (0, 1)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert got[0] == [want[0]] * 3 and got[1] == [want[1]] * 3


def test_wide_collapse_shrinks_with_width():
    lib = gpu_lib()
    w = scenes.displaced_sphere(8, 8, 1, tris=20_000)
    n = {k: g.api.plan_scene(w.prims, lib=lib, bvh_width=k, leaf_size=4).num_wide_nodes for k in (2, 4, 8)}
    assert n[2] > n[4] > n[8] > 0
    info = g.api.plan_scene(w.prims, lib=lib)
    assert info.bvh_width == 4 and info.device_bytes > 48 * info.num_components


def test_plan_rejects_bad_input():
    lib = gpu_lib()
    with pytest.raises(_abi.GrError):
        g.api.plan_scene([g.Sphere(g.Material.disney().build(), None, 1.0)], lib=lib, bvh_width=3)
    m = g.Mesh(g.Material.disney().build(), None, np.zeros((3, 3), np.float32), np.array([[0, 1, 7]]))
    with pytest.raises(_abi.GrError):
        g.api.plan_scene([m], lib=lib)


def test_plan_reports_and_bounds_the_stack_depth():
    # The build reports the wide tree's worst-case traversal stack and rejects trees
    # deeper than the traversal's 96 entries (the reference itself panics past its
    # 64-entry binary stack, geom/bvh.rs:156): spheres at x = r^k split one at a time.
    lib = gpu_lib()
    mat = g.Material.disney().build()

    def spheres(r, n):
        return [g.Sphere(mat, g.Mat.translation((float(x), 0.0, 0.0)), float(x) * 1e-3) for x in r ** np.arange(n)]

    info = g.api.plan_scene(spheres(1.05, 600), lib=lib)
    assert 0 < info.stack_depth <= 96
    assert g.api.plan_scene(scenes.cornell_spheres().prims, lib=lib).stack_depth > 0
    with pytest.raises(_abi.GrError, match="too deep"):
        g.api.plan_scene(spheres(1.1, 600), lib=lib)


def test_large_mesh_reports_the_first_bad_triangle(oracle):
    # A mesh this large is validated on threads; the error is still the first failing
    # triangle's (here a uv index at triangle 5,000 before a vertex index at 30,000).
    lib = gpu_lib()
    rng = np.random.default_rng(3)
    n = 40_000
    v = rng.random((1000, 3)).astype(np.float32)
    t = rng.integers(0, 1000, (n, 3)).astype(np.uint32)
    uv = rng.random((1000, 2)).astype(np.float32)
    tuv = rng.integers(0, 1000, (n, 3)).astype(np.uint32)
    t[30_000, 1] = 5000
    tuv[5_000, 2] = 5000
    m = g.Mesh(g.Material.disney().build(), None, v, t, uvs=uv, tri_uvs=tuv)
    for L in (lib, oracle):
        with pytest.raises(_abi.GrError, match="uv index"):
            g.api.plan_scene([m], lib=L)
    tuv[5_000, 2] = 0
    m = g.Mesh(g.Material.disney().build(), None, v, t, uvs=uv, tri_uvs=tuv)
    with pytest.raises(_abi.GrError, match="vertex index"):
        g.api.plan_scene([m], lib=lib)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _replica_worker(rank, world, port, oracle_path, q):
    import time

    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from gammaray_gb300 import replicas

    lib = _abi.Lib(oracle_path)
    w = scenes.cornell_spheres(16, 16, 1)
    st = g.Stage(w.prims, lib=lib, seed=rank)
    f = g.Film(16, 16, lib=lib)
    t0 = time.perf_counter()
    st.render(w.camera, w.integrator, f, 1 + rank)
    ms = (time.perf_counter() - t0) * 1e3 + 100.0 * rank
    t, units = replicas.aggregate(ms, 256 * (1 + rank))
    q.put((rank, ms, t, units))
    dist.destroy_process_group()


def test_replicas_two_gloo_ranks(oracle):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, oracle.path, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ms = {r: m for r, m, _, _ in out}
    for _, _, t, units in out:
        assert t == pytest.approx(max(ms.values()))
        assert units == 256 + 512
