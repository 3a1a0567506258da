"""CUDA library vs the CPU oracle on identical inputs (both through the C ABI).

Tolerances (from the parity contract):
  closest-hit (prim, component) bit-exact, except near-ties: a differing id is accepted
  only if the two hit distances agree within 1e-6 relative;
  hit distance within 1e-5 relative;
  BSDF value and pdf within 1e-5 relative (absolute floor 1e-6 for values near 0);
  images: per-path radiance agrees for >= 99% of paths, and the image relMSE between the
  two backends is far below the Monte Carlo noise.
"""
from __future__ import annotations

import zlib

import numpy as np
import pytest

import gammaray_gb300 as g
from gammaray_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu

RTOL_T = 1e-5
TIE_RTOL = 1e-6
RTOL_BSDF = 1e-5
ATOL_BSDF = 1e-6


def random_rays(n, seed, lo=-3.0, hi=3.0, target=None):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    if target is None:
        d = rng.normal(size=(n, 3))
    else:  # aim near the object so most rays hit
        d = rng.normal(size=(n, 3)) * 0.6 + (np.asarray(target) - o)
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    return np.concatenate([o, d], axis=1).astype(np.float32)


def check_hits(hg, ho):
    hit_g, hit_o = hg["prim"] >= 0, ho["prim"] >= 0
    same = (hg["prim"] == ho["prim"]) & (hg["component"] == ho["component"])
    both = hit_g & hit_o
    tie = both & ~same & (np.abs(hg["t"] - ho["t"]) <= TIE_RTOL * np.abs(ho["t"]))
    bad_id = both & ~same & ~tie
    bad_flag = hit_g != hit_o
    assert bad_flag.sum() == 0, f"{bad_flag.sum()} rays hit on one backend only"
    assert bad_id.sum() == 0, f"{bad_id.sum()} rays hit different primitives (not ties)"
    m = both & same
    np.testing.assert_allclose(hg["t"][m], ho["t"][m], rtol=RTOL_T)
    return int(both.sum()), int(tie.sum()), float((hg["t"][m] == ho["t"][m]).mean() if m.any() else 1.0)


@pytest.fixture(scope="module")
def mesh_scene(gpu, oracle):
    w = scenes.displaced_sphere(64, 64, 1)
    return w, g.Stage(w.prims, lib=gpu, environment=w.environment), g.Stage(w.prims, lib=oracle,
                                                                             environment=w.environment)


def test_trace_rays_2p20_mesh(mesh_scene):
    w, sg, so = mesh_scene
    rays = random_rays(1 << 20, 11, target=(0, 0, 0))
    hg, ho = sg.intersect(rays), so.intersect(rays)
    hits, ties, exact = check_hits(hg, ho)
    assert hits > (1 << 19)  # most rays hit the mesh
    assert exact == 1.0  # same triangle => bit-identical distance (same arithmetic)


@pytest.mark.parametrize("width", [2, 4, 8])
def test_trace_rays_widths(gpu, oracle, width):
    w = scenes.displaced_sphere(64, 64, 1, tris=20_000)
    sg = g.Stage(w.prims, lib=gpu, bvh_width=width, leaf_size=3)
    so = g.Stage(w.prims, lib=oracle)
    rays = random_rays(1 << 16, 12 + width, target=(0, 0, 0))
    check_hits(sg.intersect(rays), so.intersect(rays))


def test_trace_rays_spheres_and_naive(gpu, oracle):
    w = scenes.cornell_spheres()
    sg = g.Stage(w.prims, lib=gpu)
    so = g.Stage(w.prims, lib=oracle)
    rays = random_rays(1 << 16, 13, lo=-0.9, hi=1.9)
    hg = sg.intersect(rays)
    check_hits(hg, so.intersect(rays))
    check_hits(hg, sg.intersect_naive(rays))
    check_hits(hg, so.intersect_naive(rays))


def test_visibility(mesh_scene):
    w, sg, so = mesh_scene
    rng = np.random.default_rng(14)
    a = rng.uniform(-2.5, 2.5, (1 << 16, 3)).astype(np.float32)
    b = rng.uniform(-2.5, 2.5, (1 << 16, 3)).astype(np.float32)
    b[:16] = a[:16]  # coincident points are never visible
    pairs = np.concatenate([a, b], axis=1)
    vg, vo = sg.visibility(pairs), so.visibility(pairs)
    assert not vg[:16].any()
    assert (vg != vo).mean() < 1e-4
    assert 0.05 < vg.mean() < 0.95


def test_sample_light(gpu, oracle):
    w = scenes.displaced_sphere(64, 64, 1)
    prims = w.prims + [g.Sphere(g.Material.diffuse_light((2, 2, 2)), g.Mat.translation((2, 2, 0)), 0.5)]
    sg = g.Stage(prims, lib=gpu)
    so = g.Stage(prims, lib=oracle)
    u = np.random.default_rng(15).random((4096, 6), dtype=np.float32)
    lg, lo = sg.sample_light(u), so.sample_light(u)
    assert (lg["prim"] == lo["prim"]).all()
    for f in ("origin", "direction", "normal", "tangent", "binormal", "geom_normal"):
        np.testing.assert_allclose(lg[f], lo[f], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(lg["point_pdf"], lo["point_pdf"], rtol=1e-6)
    np.testing.assert_allclose(lg["dir_pdf"], lo["dir_pdf"], rtol=1e-5, atol=1e-6)


def random_frames(n, rng):
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    t = np.cross(nrm, rng.normal(size=(n, 3)))
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    b = np.cross(nrm, t)
    gn = nrm + 0.05 * rng.normal(size=(n, 3))
    gn /= np.linalg.norm(gn, axis=1, keepdims=True)
    fr = np.zeros(n, _abi.FRAME_DTYPE)
    fr["normal"], fr["tangent"], fr["binormal"], fr["geom_normal"] = nrm, t, b, gn
    return fr


def materials():
    D = g.Material.disney
    yield "default", D().build()
    yield "rough_aniso_sheen", D().base_color((0.8, 0.3, 0.1)).roughness(0.9).anisotropic(0.7).sheen(1.0).build()
    yield "metal", D().base_color((0.9, 0.6, 0.2)).metallic(1.0).roughness(0.2).specular_tint(0.5).build()
    yield "clearcoat", D().base_color((0.2, 0.4, 0.9)).clearcoat(1.0).clearcoat_gloss(0.7).build()
    yield "glass", D().base_color((1.0, 1.0, 1.0)).specular_trans(1.0).roughness(0.3).ior(1.5).build()
    yield "glass_exit", D().specular_trans(0.6).roughness(0.05).ior(1.8).metallic(0.2).build()
    yield "diffuse_only", D().base_color((0.5, 0.7, 0.2)).ior(1.0).build()
    yield "trans_only", D().specular_trans(1.0).ior(1.0).roughness(0.5).build()
    yield "perfect_diffuse", g.Material.diffuse()
    yield "mirror", g.Material.mirror()
    yield "light", g.Material.diffuse_light((3.0, 2.0, 1.0))


@pytest.mark.parametrize("name,mat", list(materials()))
def test_bsdf_parity(gpu, oracle, name, mat):
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    n = 1 << 15
    fr = random_frames(n, rng)
    wi = rng.normal(size=(n, 3))
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3))
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    wi, wo = wi.astype(np.float32), wo.astype(np.float32)
    for c2l in (True, False):
        fg = g.bsdf_eval(mat, fr, wi, wo, c2l, lib=gpu)
        fo = g.bsdf_eval(mat, fr, wi, wo, c2l, lib=oracle)
        np.testing.assert_allclose(fg, fo, rtol=RTOL_BSDF, atol=ATOL_BSDF)
    np.testing.assert_allclose(g.bsdf_pdf(mat, fr, wi, wo, lib=gpu), g.bsdf_pdf(mat, fr, wi, wo, lib=oracle),
                               rtol=RTOL_BSDF, atol=ATOL_BSDF)
    np.testing.assert_allclose(g.light_eval(mat, fr, wi, lib=gpu), g.light_eval(mat, fr, wi, lib=oracle),
                               rtol=0, atol=0)
    u = rng.random((n, 3), dtype=np.float32)
    sg = g.bsdf_sample(mat, fr, wi, u, True, lib=gpu)
    so = g.bsdf_sample(mat, fr, wi, u, True, lib=oracle)
    ok = np.ones(n, bool)
    for f in ("radiance", "outgoing", "emission"):
        ok &= np.isclose(sg[f], so[f], rtol=1e-4, atol=1e-5).all(axis=1)
    ok &= np.isclose(sg["pdf"], so["pdf"], rtol=1e-4, atol=1e-6)
    ok &= sg["kind"] == so["kind"]
    # Transcendentals (cos/sin/log/pow) differ by an ulp between CUDA and libm; a sample
    # right at a branch point may fall on the other side.  Allow 1 in 10^4.
    assert ok.mean() > 0.9999, f"{(~ok).sum()} of {n} samples differ"


def test_render_samples_per_path(gpu, oracle):
    for w in (scenes.cornell_spheres(48, 48, 1), scenes.displaced_sphere(48, 48, 1)):
        sg = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=7)
        so = g.Stage(w.prims, lib=oracle, environment=w.environment, seed=7)
        for pass_index in (0, 3):
            a = sg.samples(w.camera, w.integrator, w.width, w.height, pass_index)
            b = so.samples(w.camera, w.integrator, w.width, w.height, pass_index)
            np.testing.assert_array_equal(a[..., :2], b[..., :2])
            close = np.isclose(a[..., 2:], b[..., 2:], rtol=1e-4, atol=1e-5).all(axis=-1)
            assert close.mean() >= 0.99, f"{w.name}: {close.mean():.4f} of paths agree"


def test_display_color_film_bit_exact(gpu, oracle):
    w = scenes.cornell_spheres(40, 30, 1)
    films = []
    for L in (gpu, oracle):
        st = g.Stage(w.prims, lib=L, seed=3)
        f = g.Film(40, 30, lib=L)
        st.render(w.camera, g.DisplayColorIntegrator(), f, 3)
        films.append(f.read())
    (ag, wg), (ao, wo) = films
    np.testing.assert_array_equal(wg, wo)  # weights depend on the jitter only
    same = (ag == ao).all(axis=-1)
    assert same.mean() > 0.999


def test_image_statistics(gpu, oracle):
    w = scenes.cornell_spheres(64, 64, 16)
    imgs = []
    for L in (gpu, oracle):
        st = g.Stage(w.prims, lib=L, seed=5)
        f = g.Film(64, 64, lib=L)
        st.render(w.camera, w.integrator, f, 16)
        imgs.append(f.resolve())
    a, b = imgs
    rel_mse = float(np.mean((a - b) ** 2) / np.mean(b ** 2))
    assert rel_mse < 1e-3, rel_mse


def test_converged_render_within_rel_mse(gpu, oracle):
    # A converged GPU render against the oracle's 4096-spp render of the same scene, with
    # independent random streams (different seeds): relMSE <= 1e-3.  On this scene one
    # render's relMSE is about 1.05 / spp, so two independent 4096-spp renders differ
    # by about 5e-4.
    w = scenes.cornell_spheres(48, 48, 4096)
    imgs = []
    for L, seed in ((gpu, 21), (oracle, 22)):
        st = g.Stage(w.prims, lib=L, seed=seed)
        f = g.Film(48, 48, lib=L)
        st.render(w.camera, w.integrator, f, 4096)
        imgs.append(f.resolve())
    a, b = imgs
    rel_mse = float(np.mean((a - b) ** 2) / np.mean(b ** 2))
    assert rel_mse <= 1e-3, rel_mse


def _exr_lines(b, W, H):
    """Decodes an ExrWriter file (render/exr.rs:138-199): the magic and version, the line
    offset table after the header, and per line its y, byte count and B, G, R float32
    planes.  Returns the image as (H, W, 3) RGB with row 0 first, like Film::pixels."""
    import struct

    assert struct.unpack("<ii", b[:8]) == (20000630, 2)
    line = 8 + W * 12
    table = len(b) - H * line - 8 * H
    offsets = [struct.unpack("<Q", b[table + 8 * k:table + 8 * k + 8])[0] for k in range(H)]
    assert offsets == [len(b) - H * line + k * line for k in range(H)]
    img = np.empty((H, W, 3), np.float32)
    for y, off in enumerate(offsets):
        assert struct.unpack("<iI", b[off:off + 8]) == (y, line - 8)
        planes = np.frombuffer(b[off + 8:off + line], "<f4").reshape(3, W)
        img[H - 1 - y] = planes[::-1].T  # B, G, R planes; line y holds film row H - 1 - y
    return img


def test_exr_matches_oracle(gpu, oracle, tmp_path):
    # A varied display-colour image of odd width: the GPU's file is the oracle's, byte for
    # byte (header, offset table, and every line's B, G, R planes, rows flipped), and it
    # decodes to the GPU film's own resolve.
    W, H = 21, 13
    w = scenes.cornell_spheres(W, H, 1)
    out = []
    for L, name in ((gpu, "g.exr"), (oracle, "o.exr")):
        st = g.Stage(w.prims, lib=L, seed=3)
        f = g.Film(W, H, lib=L)
        st.render(w.camera, g.DisplayColorIntegrator(), f, 2)
        f.write_exr(str(tmp_path / name))
        out.append(((tmp_path / name).read_bytes(), f.resolve()))
    (bg, rg), (bo, ro) = out
    assert len(np.unique(rg.reshape(-1, 3), axis=0)) > 3  # varied, so a misplaced line shows
    np.testing.assert_array_equal(_exr_lines(bg, W, H), rg)
    np.testing.assert_array_equal(_exr_lines(bo, W, H), ro)
    assert bg == bo


def test_exr_adds_the_light_tracing_splats(gpu, tmp_path):
    # A BDPT film with light-tracing splats: every EXR line decodes to the film's resolve
    # (accum / weight + splat / passes), bit for bit.
    W, H = 19, 11
    w = scenes.cornell_spheres(W, H, 1)
    st = g.Stage(w.prims, lib=gpu, seed=8)
    f = g.Film(W, H, lib=gpu)
    st.render(w.camera, g.BdptIntegrator(max_depth=8, mis=1, light_tracing=1), f, 3)
    assert f.read_splat().sum() > 0
    f.write_exr(str(tmp_path / "s.exr"))
    np.testing.assert_array_equal(_exr_lines((tmp_path / "s.exr").read_bytes(), W, H), f.resolve())


def test_step_budget_is_reported(gpu, monkeypatch):
    # A traversal step budget that the rays exceed (set on the host, GR_STEP_BUDGET, read at
    # scene creation; no GPU fault): the render returns GR_ERR_TIMEOUT naming the budget,
    # and a render of a scene with the normal budget then works.
    w = scenes.cornell_spheres(32, 32, 1)
    monkeypatch.setenv("GR_STEP_BUDGET", "1")
    st = g.Stage(w.prims, lib=gpu, seed=2)
    monkeypatch.delenv("GR_STEP_BUDGET")
    f = g.Film(32, 32, lib=gpu)
    with pytest.raises(_abi.GrError) as e:
        st.render(w.camera, w.integrator, f, 1)
    assert e.value.status == 5 and "step budget" in str(e.value)
    ok = g.Stage(w.prims, lib=gpu, seed=2)
    f2 = g.Film(32, 32, lib=gpu)
    ok.render(w.camera, w.integrator, f2, 1)
    assert f2.read()[1].sum() > 0


@pytest.mark.parametrize("scene", ["cornell", "displaced", "displaced_env_spheres", "no_lights"])
def test_bdpt_samples_per_path(gpu, oracle, scene):
    if scene == "cornell":
        w = scenes.cornell_spheres(40, 40, 1)
        prims, env, integ = w.prims, w.environment, g.BdptIntegrator()
    elif scene == "displaced":
        w = scenes.displaced_sphere(40, 40, 1, bdpt=True)
        prims, env, integ = w.prims, (0, 0, 0), w.integrator
    elif scene == "displaced_env_spheres":
        w = scenes.displaced_sphere(40, 40, 1, bdpt=True, tris=20_000)
        prims = w.prims + [g.Sphere(g.Material.diffuse_light((3, 3, 3)), g.Mat.translation((1.5, 1.0, 0)), 0.3),
                           g.Sphere(g.Material.mirror(), g.Mat.translation((-1.5, -0.6, 0.5)), 0.5)]
        env, integ = w.environment, w.integrator
    else:
        w = scenes.cornell_spheres(40, 40, 1)
        prims = [p for p in w.prims if not p.material.has_light()]
        env, integ = (0.5, 0.5, 0.5), g.BdptIntegrator(max_depth=8)
    sg = g.Stage(prims, lib=gpu, environment=env, seed=21)
    so = g.Stage(prims, lib=oracle, environment=env, seed=21)
    for pass_index in (0, 5):
        a = sg.samples(w.camera, integ, 40, 40, pass_index)
        b = so.samples(w.camera, integ, 40, 40, pass_index)
        np.testing.assert_array_equal(a[..., :2], b[..., :2])
        close = np.isclose(a[..., 2:], b[..., 2:], rtol=1e-4, atol=1e-5).all(axis=-1)
        assert close.mean() >= 0.99, f"{scene}: {close.mean():.4f} of paths agree"
        assert np.isfinite(a[..., 2:]).all()


def test_bdpt_image_statistics(gpu, oracle):
    w = scenes.cornell_spheres(48, 48, 8)
    imgs = []
    for L in (gpu, oracle):
        st = g.Stage(w.prims, lib=L, seed=6)
        f = g.Film(48, 48, lib=L)
        st.render(w.camera, g.BdptIntegrator(), f, 8)
        imgs.append(f.resolve())
    a, b = imgs
    rel_mse = float(np.mean((a - b) ** 2) / np.mean(b ** 2))
    assert rel_mse < 1e-3, rel_mse
    assert gpu.backend == "cuda-sm_103a"


def test_bdpt_groups_do_not_change_the_film(gpu, monkeypatch):
    # Paths in flight only decide how passes are grouped: random streams are keyed by
    # pass, and each path's strategies are summed in loop order, so with MIS (and no
    # light-tracing splats, whose atomics add in any order) the film is bit-identical
    # whether a render runs as one group or as many.
    w = scenes.cornell_spheres(32, 32, 6)
    st = g.Stage(w.prims, lib=gpu, seed=12)
    films = []
    for paths in (None, "1024"):
        if paths is None:
            monkeypatch.delenv("GR_BDPT_PATHS_IN_FLIGHT", raising=False)
        else:
            monkeypatch.setenv("GR_BDPT_PATHS_IN_FLIGHT", paths)  # one 32x32 pass per group
        st._pass = 0
        f = g.Film(32, 32, lib=gpu)
        st.render(w.camera, g.BdptIntegrator(max_depth=8, mis=1), f, 6)
        films.append(f.read())
    np.testing.assert_array_equal(films[0][0], films[1][0])
    np.testing.assert_array_equal(films[0][1], films[1][1])


def test_pt_groups_do_not_change_the_film(gpu, monkeypatch):
    # The path tracer's film is bit-identical whether the passes run as one group of
    # paths in flight or one pass per group (the deterministic gather adds them in pass
    # order either way).
    w = scenes.displaced_sphere(40, 40, 5)
    st = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=4)
    films = []
    for paths in (None, "1600"):
        if paths is None:
            monkeypatch.delenv("GR_PATHS_IN_FLIGHT", raising=False)
        else:
            monkeypatch.setenv("GR_PATHS_IN_FLIGHT", paths)
        st._pass = 0
        f = g.Film(40, 40, lib=gpu)
        st.render(w.camera, w.integrator, f, 5)
        films.append(f.read())
    np.testing.assert_array_equal(films[0][0], films[1][0])
    np.testing.assert_array_equal(films[0][1], films[1][1])


@pytest.mark.parametrize("bdpt", [False, True])
def test_chunked_film_gather_equals_pass_by_pass(gpu, monkeypatch, bdpt):
    # A 768x512 image has 1,024 film tiles, more than the gather's resident blocks, so
    # 16 passes in one group are added in ordered 8-pass chunks over all tiles; one pass
    # per group adds each pass with one block per tile.  Both sum every pixel in pass
    # order: the films are bit-identical.
    width, height, spp = 768, 512, 16
    w = scenes.displaced_sphere(width, height, spp, bdpt=bdpt)
    st = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=9)
    integ = g.BdptIntegrator(max_depth=6, mis=1) if bdpt else w.integrator
    env = "GR_BDPT_PATHS_IN_FLIGHT" if bdpt else "GR_PATHS_IN_FLIGHT"
    films = []
    for paths in (None, str(width * height)):
        if paths is None:
            monkeypatch.delenv(env, raising=False)
        else:
            monkeypatch.setenv(env, paths)
        st._pass = 0
        f = g.Film(width, height, lib=gpu)
        st.render(w.camera, integ, f, spp)
        films.append(f.read())
    assert films[0][1].min() > 0
    np.testing.assert_array_equal(films[0][1], films[1][1])
    np.testing.assert_array_equal(films[0][0], films[1][0])


def test_film_chunk_wait_runs_out_and_is_reported(gpu, monkeypatch):
    # A chunk of the film gather waits (bounded) for its tile's previous chunk.  With
    # GR_FILM_WAIT_TEST set, the first chunk's items never run, so no flag is ever set and
    # every later item's wait runs out (no fault): the render returns GR_ERR_TIMEOUT, and
    # the next render on the same scene works and gives the film it should.
    width, height, spp = 768, 512, 16
    w = scenes.displaced_sphere(width, height, spp)
    st = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=9)
    monkeypatch.setenv("GR_FILM_WAIT_TEST", "1")
    f = g.Film(width, height, lib=gpu)
    with pytest.raises(_abi.GrError) as e:
        st.render(w.camera, w.integrator, f, spp)
    assert e.value.status == 5 and "wait between pass chunks" in str(e.value)
    monkeypatch.delenv("GR_FILM_WAIT_TEST")
    films = []
    for paths in (None, str(width * height)):  # chunked, then one pass per group
        if paths is None:
            monkeypatch.delenv("GR_PATHS_IN_FLIGHT", raising=False)
        else:
            monkeypatch.setenv("GR_PATHS_IN_FLIGHT", paths)
        st._pass = 0
        f = g.Film(width, height, lib=gpu)
        st.render(w.camera, w.integrator, f, spp)
        films.append(f.read())
    np.testing.assert_array_equal(films[0][1], films[1][1])
    np.testing.assert_array_equal(films[0][0], films[1][0])


def test_sync_check_reports_a_slow_launch(gpu):
    # GR_SYNC_CHECK bounds every host wait of a render.  With a limit no launch can meet,
    # the render returns GR_ERR_TIMEOUT naming the kernel, the work in flight finishes
    # normally, and the context stays usable.  (A subprocess: the limit is read once.)
    import os
    import subprocess
    import sys

    code = """
import torch
import gammaray_gb300 as g
from gammaray_gb300 import _abi, scenes
w = scenes.displaced_sphere(256, 256, 4)
st = g.Stage(w.prims, environment=w.environment)
f = g.Film(256, 256)
try:
    st.render(w.camera, w.integrator, f, 4)
    print("NO_TIMEOUT")
except _abi.GrError as e:
    print("TIMEOUT", e)
torch.cuda.synchronize()
print("OK", torch.ones(1024, device="cuda").sum().item())
"""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, GR_SYNC_CHECK="1e-9", PYTHONPATH=root)
    r = subprocess.run([sys.executable, "-c", code], env=env, cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "TIMEOUT" in r.stdout and "did not finish" in r.stdout, r.stdout
    assert "OK 1024.0" in r.stdout, r.stdout


@pytest.mark.parametrize("at", [1, 3, 6, 9, 12, 15])
def test_allocation_refusal_is_reported_and_recovered(gpu, at):
    # Host-side fault injection (GR_FAIL_ALLOC_AT=k: the k-th device allocation reports
    # out of memory, once).  Wherever it lands (scene creation, film, the render's path
    # state), the call fails with an error, nothing crashes, and the same work then
    # succeeds in the same process.  (A subprocess: the setting is read once.)
    import os
    import subprocess
    import sys

    code = """
import numpy as np
import gammaray_gb300 as g
from gammaray_gb300 import _abi, scenes
w = scenes.cornell_spheres(32, 32, 2)
def attempt():
    st = g.Stage(w.prims, environment=w.environment, seed=3)
    f = g.Film(32, 32)
    st.render(w.camera, w.integrator, f, 2)
    return f.resolve()
try:
    attempt()
    print("FIRST_OK")
except _abi.GrError as e:
    print("FIRST_ERROR", e)
img = attempt()
print("RECOVERED", bool(np.isfinite(img).all()), float(img.mean()) > 0.0)
"""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, GR_FAIL_ALLOC_AT=str(at), PYTHONPATH=root)
    r = subprocess.run([sys.executable, "-c", code], env=env, cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "FIRST_ERROR" in r.stdout and "memory" in r.stdout.lower(), r.stdout
    assert "RECOVERED True True" in r.stdout, r.stdout


def test_bdpt_counts_shadow_rays(gpu):
    w = scenes.cornell_spheres(32, 32, 2)
    st = g.Stage(w.prims, lib=gpu, seed=1)
    f = g.Film(32, 32, lib=gpu)
    st.render(w.camera, g.BdptIntegrator(), f, 2)
    s = st.last_stats()
    assert s.samples == 2 * 32 * 32 and s.extension_rays > s.samples and s.shadow_rays > 0


@pytest.mark.parametrize("lt", [0, 1])
@pytest.mark.parametrize("scene", ["cornell", "displaced_env_spheres"])
def test_bdpt_mis_samples_per_path(gpu, oracle, scene, lt):
    # Power-heuristic weights per path against the oracle (the mirror sphere exercises
    # the delta-vertex rules); light-tracing splats are not part of per-path samples.
    if scene == "cornell":
        w = scenes.cornell_spheres(40, 40, 1)
        prims, env = w.prims, w.environment
    else:
        w = scenes.displaced_sphere(40, 40, 1, bdpt=True, tris=20_000)
        prims = w.prims + [g.Sphere(g.Material.diffuse_light((3, 3, 3)), g.Mat.translation((1.5, 1.0, 0)), 0.3),
                           g.Sphere(g.Material.mirror(), g.Mat.translation((-1.5, -0.6, 0.5)), 0.5)]
        env = w.environment
    integ = g.BdptIntegrator(max_depth=10, mis=1, light_tracing=lt)
    sg = g.Stage(prims, lib=gpu, environment=env, seed=23)
    so = g.Stage(prims, lib=oracle, environment=env, seed=23)
    a = sg.samples(w.camera, integ, 40, 40, 3)
    b = so.samples(w.camera, integ, 40, 40, 3)
    np.testing.assert_array_equal(a[..., :2], b[..., :2])
    close = np.isclose(a[..., 2:], b[..., 2:], rtol=1e-4, atol=1e-5).all(axis=-1)
    assert close.mean() >= 0.99, f"{scene}: {close.mean():.4f} of paths agree"
    assert np.isfinite(a[..., 2:]).all()


def test_bdpt_light_tracing_film_parity(gpu, oracle):
    # The same light-tracing terms on both sides; the GPU adds them with atomics, so only
    # the order of the additions (and BSDF ulps) differs.
    w = scenes.cornell_spheres(40, 40, 1)
    out = []
    for L in (gpu, oracle):
        st = g.Stage(w.prims, lib=L, seed=5)
        f = g.Film(40, 40, lib=L)
        st.render(w.camera, g.BdptIntegrator(max_depth=10, mis=1, light_tracing=1), f, 2)
        out.append((f.read(), f.read_splat(), f.resolve(), f.passes()))
    (ga, gw), gs, gr, gp = out[0]
    (oa, ow), os_, orr, op = out[1]
    assert gp == op == 2
    assert gs.sum() > 0
    rel = lambda x, y: float(np.sqrt(np.mean((x - y) ** 2) / np.mean(y ** 2)))
    assert rel(gs, os_) < 1e-3, rel(gs, os_)
    assert rel(ga, oa) < 1e-3 and rel(gw, ow) < 1e-6
    assert rel(gr, orr) < 1e-3


def test_bdpt_mis_unbiased_against_pt(gpu):
    # MIS + light tracing on the GPU converges to the path tracer's image away from the
    # directly visible light and the image edge (see test_oracle.far_from_bright).
    from test_oracle import far_from_bright

    w = scenes.cornell_spheres(64, 64, 1)
    st = g.Stage(w.prims, lib=gpu, seed=4)
    fp, fb = g.Film(64, 64, lib=gpu), g.Film(64, 64, lib=gpu)
    st.render(w.camera, g.PathTracerIntegrator(), fp, 4096)
    st.render(w.camera, g.BdptIntegrator(mis=1, light_tracing=1), fb, 256)
    pt, b = fp.resolve(), fb.resolve()
    keep = far_from_bright(pt)
    ref, got = float(pt[keep].mean()), float(b[keep].mean())
    assert abs(got - ref) / ref < 0.01, (ref, got)
    # 8x8-pixel block means agree to within the noise of both images
    k = keep.reshape(8, 8, 8, 8).transpose(0, 2, 1, 3).reshape(64, 64).all(axis=1)
    bp = pt.reshape(8, 8, 8, 8, 3).mean(axis=(1, 3)).reshape(64, 3)[k]
    bb = b.reshape(8, 8, 8, 8, 3).mean(axis=(1, 3)).reshape(64, 3)[k]
    assert len(bp) >= 8
    assert float(np.mean((bb - bp) ** 2) / np.mean(bp ** 2)) < 2e-3
