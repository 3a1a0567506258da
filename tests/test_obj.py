"""OBJ ingest (Mesh::from_obj, geom/mesh.rs:61-160) on the CPU: the parser rules the
reference relies on (object-local indices, polygon fans, skipped statements, errors
with line numbers) and from_obj's uv / shading-normal fallbacks.  A mesh loaded from
OBJ renders exactly like the same mesh built from arrays (oracle)."""
from __future__ import annotations

import os

import numpy as np
import pytest

import gammaray_gb300 as g
from gammaray_gb300 import _abi, obj

CUBE = """\
# unit cube, quads, with uvs and normals
mtllib cube.mtl
o cube
v -1 -1 -1
v  1 -1 -1
v  1  1 -1
v -1  1 -1
v -1 -1  1
v  1 -1  1
v  1  1  1
v -1  1  1
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 -1
vn 0 0 1
vn 0 -1 0
vn 0 1 0
vn -1 0 0
vn 1 0 0
usemtl grey
s off
f 1/1/1 4/4/1 3/3/1 2/2/1
f 5/1/2 6/2/2 7/3/2 8/4/2
f 1/1/3 2/2/3 6/3/3 5/4/3
f 4/1/4 8/2/4 7/3/4 3/4/4
f 1/1/5 5/2/5 8/3/5 4/4/5
f 2/1/6 3/2/6 7/3/6 6/4/6
"""


def write(tmp_path, text, name="m.obj"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_quads_become_fans():
    objs = obj.parse_obj(CUBE)
    assert len(objs) == 1 and objs[0].name == "cube"
    tris = objs[0].triangles
    assert len(tris) == 12
    # f 1/1/1 4/4/1 3/3/1 2/2/1 -> (1,4,3), (1,3,2), 0-based
    assert [t[0] for t in tris[0]] == [0, 3, 2] and [t[0] for t in tris[1]] == [0, 2, 1]
    assert tris[0][1] == (3, 3, 0)


def test_pentagon_fan_and_skipped_statements():
    text = "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv -1 0.5 0\ng a\ns 1\nl 1 2\np 3\nf 1 2 3 4 5\n"
    tris = obj.parse_obj(text)[0].triangles
    assert [[v[0] for v in t] for t in tris] == [[0, 1, 2], [0, 2, 3], [0, 3, 4]]


def test_objects_have_local_indices_and_offsets():
    text = ("o a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n"
            "o b\nv 0 0 1\nv 1 0 1\nv 0 1 1\nf 4 5 6\nf -3 -2 -1\n")
    objs = obj.parse_obj(text)
    assert [o.name for o in objs] == ["a", "b"]
    assert [v[0] for v in objs[1].triangles[0]] == [0, 1, 2]
    assert [v[0] for v in objs[1].triangles[1]] == [0, 1, 2]
    v, t, n, tn, uv, tuv = obj.mesh_arrays(objs)
    assert t.tolist() == [[0, 1, 2], [3, 4, 5], [3, 4, 5]]


def test_uv_and_normal_fallbacks():
    text = ("v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0.25 0.5\nvn 0 0 1\nvn 0 0 0\n"
            "f 1/1/1 2/1/1 3/1/1\n"  # complete: uses its uvs and normals
            "f 1 2 3\n"  # no uvs, no normals
            "f 1/1/1 2/1/2 3/1/1\n"  # one degenerate normal
            "f 1//1 2//1 3//1\n")  # normals without uvs
    v, t, n, tn, uv, tuv = obj.mesh_arrays(obj.parse_obj(text))
    assert tuv[0].tolist() == [0, 0, 0]
    # each triangle without a complete uv set gets its own fresh zero uv
    assert tuv[1].tolist() == [1, 1, 1] and tuv[3].tolist() == [2, 2, 2]
    assert uv.tolist() == [[0.25, 0.5], [0.0, 0.0], [0.0, 0.0]]
    assert tn[0].tolist() == [0, 0, 0] and tn[3].tolist() == [0, 0, 0]
    assert tn[1].tolist() == [_abi.NO_INDEX] * 3 and tn[2].tolist() == [_abi.NO_INDEX] * 3


def test_normals_are_transformed_and_normalised(tmp_path):
    text = "v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 2\nvn 0 0 0\nf 1//1 2//1 3//1\n"
    m = g.Mesh.from_obj(g.Material.disney().build(), None, write(tmp_path, text))
    assert m.normals.tolist() == [[0.0, 0.0, 1.0], [0.0, 0.0, 0.0]]
    m2 = g.Mesh.from_obj(g.Material.disney().build(), g.Mat.scale(2.0), write(tmp_path, text))
    assert np.allclose(m2.vertices[1], [2, 0, 0]) and np.allclose(m2.normals[0], [0, 0, 1])


@pytest.mark.parametrize("text,where", [("v 0 0\n", 1), ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n", 4),
                                        ("v 0 0 0\nf 1 2\n", 2), ("v 0 0 0\nbogus 1\n", 2),
                                        ("v 0 0 0\nv 0 0 0\nv 0 0 0\nf 1/2 2 3\n", 4), ("vn 0 0 x\n", 1)])
def test_parse_errors_name_the_line(tmp_path, text, where):
    with pytest.raises(obj.ObjError, match=f"OBJ parse error at line {where}:"):
        g.Mesh.from_obj(g.Material.disney().build(), None, write(tmp_path, text))


def test_missing_file():
    with pytest.raises(obj.ObjError, match="Couldn't open OBJ file"):
        g.Mesh.from_obj(g.Material.disney().build(), None, "/nonexistent/x.obj")


def test_obj_renders_like_arrays(oracle, tmp_path):
    mat = g.Material.disney().base_color((0.6, 0.5, 0.4)).roughness(0.4).build()
    xf = g.Mat.translation((0, 0, -4))
    a = g.Mesh.from_obj(mat, xf, write(tmp_path, CUBE))
    objs = obj.parse_obj(CUBE)
    v, t, n, tn, uv, tuv = obj.mesh_arrays(objs)
    b = g.Mesh(mat, xf, v, t, normals=n, tri_normals=tn, uvs=uv, tri_uvs=tuv)
    light = g.Sphere(g.Material.diffuse_light((4, 4, 4)), g.Mat.translation((2, 3, 0)), 0.5)
    cam = g.Camera.with_fov(40.0)
    films = []
    for mesh in (a, b):
        st = g.Stage([mesh, light], lib=oracle, environment=(0.1, 0.1, 0.1))
        films.append(st.samples(cam, g.PathTracerIntegrator(max_depth=4), 24, 24))
    assert np.array_equal(films[0], films[1])


REF_CONE = os.path.join(os.sep, "root", "reference", "cone.obj")


@pytest.mark.skipif(not os.path.exists(REF_CONE), reason="the reference's sample mesh is not on this machine")
def test_reference_cone_loads():
    m = g.Mesh.from_obj(g.Material.disney().build(), None, REF_CONE)
    # 20 side triangles plus the 20-gon base as an 18-triangle fan
    assert m.num_components() == 38
    assert np.isfinite(m.vertices).all()


def sphere_obj(rings=12, segments=16):
    """A latitude-longitude sphere as OBJ text: quad bands, triangle fans at the poles,
    per-vertex normals and uvs (shading normals and uvs both reach the renderer)."""
    lines = ["o ball"]
    for r in range(rings + 1):
        th = np.pi * r / rings
        for s in range(segments):
            ph = 2 * np.pi * s / segments
            x, y, z = np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)
            lines.append(f"v {x:.6f} {y:.6f} {z:.6f}")
            lines.append(f"vn {x:.6f} {y:.6f} {z:.6f}")
            lines.append(f"vt {s / segments:.6f} {r / rings:.6f}")
    idx = lambda r, s: r * segments + (s % segments) + 1
    for r in range(rings):
        for s in range(segments):
            a, b, c, d = idx(r, s), idx(r, s + 1), idx(r + 1, s + 1), idx(r + 1, s)
            if r == 0:
                lines.append(f"f {a}/{a}/{a} {c}/{c}/{c} {d}/{d}/{d}")
            elif r == rings - 1:
                lines.append(f"f {a}/{a}/{a} {b}/{b}/{b} {d}/{d}/{d}")
            else:
                lines.append(f"f {a}/{a}/{a} {b}/{b}/{b} {c}/{c}/{c} {d}/{d}/{d}")
    return "\n".join(lines) + "\n"


@pytest.mark.gpu
def test_obj_meshes_render_per_path_on_gpu(gpu, oracle, tmp_path):
    # OBJ meshes (quads and polygons fanned, shading normals, uvs) traced and shaded on
    # the GPU: every path's film position equal to the oracle's, and at least 99% of the
    # paths' radiance within 1e-4 (the per-path bar of the other scenes).
    metal = g.Material.disney().base_color((0.9, 0.7, 0.5)).metallic(1.0).roughness(0.3).build()
    grey = g.Material.disney().base_color((0.6, 0.5, 0.4)).roughness(0.4).build()
    ball = g.Mesh.from_obj(metal, g.Mat.translation((0.8, 0.0, -4.0)), write(tmp_path, sphere_obj(), "ball.obj"))
    cube = g.Mesh.from_obj(grey, g.Mat.translation((-1.2, -0.5, -5.0)), write(tmp_path, CUBE))
    assert ball.num_components() == 2 * 16 + 2 * 10 * 16  # fans at the poles, quads between
    light = g.Sphere(g.Material.diffuse_light((4, 4, 4)), g.Mat.translation((2, 3, 0)), 0.5)
    prims = [ball, cube, light]
    cam = g.Camera.with_fov(40.0)
    integ = g.PathTracerIntegrator(max_depth=6)
    sg = g.Stage(prims, lib=gpu, environment=(0.1, 0.1, 0.1), seed=3)
    so = g.Stage(prims, lib=oracle, environment=(0.1, 0.1, 0.1), seed=3)
    for pass_index in (0, 2):
        a = sg.samples(cam, integ, 48, 40, pass_index)
        b = so.samples(cam, integ, 48, 40, pass_index)
        np.testing.assert_array_equal(a[..., :2], b[..., :2])
        close = np.isclose(a[..., 2:], b[..., 2:], rtol=1e-4, atol=1e-5).all(axis=-1)
        assert close.mean() >= 0.99, f"{close.mean():.4f} of paths agree"
        assert (b[..., 2:] > 0).any()  # the meshes are lit
