"""OBJ mesh ingest: Mesh::from_obj (geom/mesh.rs:61-160) over a Wavefront OBJ parser.

The reference parses with the `wavefront_obj` crate (5.1.0, a Cargo dependency that is
not vendored with the reference).  This module restates the part of that parser's
behaviour that Mesh::from_obj relies on:

  - `o name` starts a new object; geometry before the first `o` forms an unnamed one.
    Each object has its own vertex, texture-vertex and normal lists, and face indices
    are made object-local: the OBJ file's 1-based, file-global index i becomes
    i - 1 - (count defined in earlier objects).  Negative indices count back from the
    last element defined so far (OBJ's relative form).
  - `v x y z [w]`, `vt u [v [w]]` (missing v is 0) and `vn x y z` are read as f64 and
    converted to f32 by Mesh::from_obj (`v.x as f32`).
  - `f` takes vertex references `v`, `v/t`, `v//n` or `v/t/n`.  A polygon of n > 3
    vertices becomes the fan (0, k, k+1), k = 1..n-2.
  - `l` / `p` (lines, points), `g`, `s`, `usemtl` and `mtllib` carry no triangles and
    are skipped, as from_obj keeps only Primitive::Triangle shapes.
  - Malformed lines raise an error naming the line, as `OBJ parse error at line N: ...`.

Mesh::from_obj then, per object (mesh.rs:96-150):
  - transforms points by the xform;
  - transforms normals by the inverse transpose and normalises them, unless they are
    nearly zero;
  - uses a triangle's uv indices only when all three are given, else gives it one fresh
    zero uv;
  - uses its normal indices only when all three are given and none of those normals is
    nearly zero, else marks it for the geometric normal (GR_NO_INDEX).
"""
from __future__ import annotations

import numpy as np

from . import _abi


class ObjError(ValueError):
    pass


class _Obj:
    def __init__(self, name: str):
        self.name = name
        self.vertices: list[tuple[float, float, float]] = []
        self.tex: list[tuple[float, float]] = []
        self.normals: list[tuple[float, float, float]] = []
        self.triangles: list[tuple[tuple[int, int | None, int | None], ...]] = []


def _floats(parts, lo, hi, line_no, what):
    if not (lo <= len(parts) <= hi):
        raise ObjError(f"OBJ parse error at line {line_no}: {what} expects {lo} to {hi} numbers")
    try:
        return [float(p) for p in parts]
    except ValueError:
        raise ObjError(f"OBJ parse error at line {line_no}: bad number in {what}") from None


def _index(tok: str, defined_before: int, defined_now: int, line_no: int) -> int:
    """One OBJ index (1-based, file-global, or negative = relative) -> object-local."""
    try:
        i = int(tok)
    except ValueError:
        raise ObjError(f"OBJ parse error at line {line_no}: bad index {tok!r}") from None
    if i > 0:
        local = i - 1 - defined_before
    elif i < 0:
        local = defined_now + i
    else:
        raise ObjError(f"OBJ parse error at line {line_no}: index 0")
    if not (0 <= local < defined_now):
        raise ObjError(f"OBJ parse error at line {line_no}: index {tok} out of range")
    return local


def parse_obj(text: str) -> list[_Obj]:
    """Objects of an OBJ text, with object-local triangle indices (see module doc)."""
    objs: list[_Obj] = []
    cur: _Obj | None = None
    before = [0, 0, 0]  # vertices, texture vertices, normals of earlier objects

    def current() -> _Obj:
        nonlocal cur
        if cur is None:
            cur = _Obj("")
            objs.append(cur)
        return cur

    for line_no, raw in enumerate(text.splitlines(), start=1):
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        parts = line.split()
        key, args = parts[0], parts[1:]
        if key == "o":
            if cur is not None:
                before = [before[0] + len(cur.vertices), before[1] + len(cur.tex), before[2] + len(cur.normals)]
            cur = _Obj(" ".join(args))
            objs.append(cur)
        elif key == "v":
            x = _floats(args, 3, 4, line_no, "v")
            current().vertices.append((x[0], x[1], x[2]))
        elif key == "vt":
            x = _floats(args, 1, 3, line_no, "vt")
            current().tex.append((x[0], x[1] if len(x) > 1 else 0.0))
        elif key == "vn":
            x = _floats(args, 3, 3, line_no, "vn")
            current().normals.append((x[0], x[1], x[2]))
        elif key == "f":
            o = current()
            if len(args) < 3:
                raise ObjError(f"OBJ parse error at line {line_no}: a face needs at least 3 vertices")
            refs = []
            for a in args:
                f = a.split("/")
                if len(f) > 3 or f[0] == "":
                    raise ObjError(f"OBJ parse error at line {line_no}: bad vertex reference {a!r}")
                v = _index(f[0], before[0], len(o.vertices), line_no)
                t = _index(f[1], before[1], len(o.tex), line_no) if len(f) > 1 and f[1] != "" else None
                n = _index(f[2], before[2], len(o.normals), line_no) if len(f) > 2 and f[2] != "" else None
                refs.append((v, t, n))
            for k in range(1, len(refs) - 1):
                o.triangles.append((refs[0], refs[k], refs[k + 1]))
        elif key in ("l", "p", "g", "s", "usemtl", "mtllib"):
            continue
        else:
            raise ObjError(f"OBJ parse error at line {line_no}: unknown statement {key!r}")
    return objs


def mesh_arrays(objs: list[_Obj]):
    """Mesh::from_obj's vertex / normal / uv lists and per-triangle indices
    (mesh.rs:96-150), before the xform.  Returns (vertices, triangles, normals,
    tri_normals, uvs, tri_uvs) as numpy arrays; tri_normals rows of GR_NO_INDEX select
    the geometric normal."""
    eps = np.finfo(np.float32).eps
    verts, norms, uvs, tris, tri_n, tri_t = [], [], [], [], [], []
    for o in objs:
        off, noff, toff = len(verts), len(norms), len(uvs)
        verts.extend(o.vertices)
        norms.extend(o.normals)
        uvs.extend(o.tex)
        nz = [float(np.float32(x) * np.float32(x) + np.float32(y) * np.float32(y) + np.float32(z) * np.float32(z)) < eps
              for (x, y, z) in o.normals]
        for a, b, c in o.triangles:
            tris.append((off + a[0], off + b[0], off + c[0]))
            if a[1] is not None and b[1] is not None and c[1] is not None:
                tri_t.append((toff + a[1], toff + b[1], toff + c[1]))
            else:
                uvs.append((0.0, 0.0))
                z = len(uvs) - 1
                tri_t.append((z, z, z))
            if (a[2] is not None and b[2] is not None and c[2] is not None
                    and not (nz[a[2]] or nz[b[2]] or nz[c[2]])):
                tri_n.append((noff + a[2], noff + b[2], noff + c[2]))
            else:
                tri_n.append((_abi.NO_INDEX,) * 3)
    f32 = np.float32
    return (np.asarray(verts, f32).reshape(-1, 3), np.asarray(tris, np.uint32).reshape(-1, 3),
            np.asarray(norms, f32).reshape(-1, 3), np.asarray(tri_n, np.uint32).reshape(-1, 3),
            np.asarray(uvs, f32).reshape(-1, 2), np.asarray(tri_t, np.uint32).reshape(-1, 3))


def load_obj(material, xf, path: str):
    """Mesh::from_obj(material, xf_mat, path) (mesh.rs:61-160)."""
    from .api import Mat, Mesh

    try:
        with open(path, "rb") as f:
            data = f.read()
    except OSError as e:
        raise ObjError(f"Couldn't open OBJ file: {e}") from None
    try:
        text = data.decode("utf-8")
    except UnicodeDecodeError as e:
        raise ObjError(f"Couldn't read OBJ file: {e}") from None
    v, t, n, tn, uv, tuv = mesh_arrays(parse_obj(text))
    if len(t) == 0:
        raise ObjError("OBJ file has no triangles")
    normals = n if len(n) else None
    # from_obj always builds an Xform, so normals are normalised even without a matrix.
    return Mesh(material, xf if xf is not None else Mat.identity(), v, t, normals=normals,
                tri_normals=tn if normals is not None else None, uvs=uv, tri_uvs=tuv)
