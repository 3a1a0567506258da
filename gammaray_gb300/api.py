"""Host-side mirror of the reference's public Rust API, over the C ABI.

A user of the reference writes (src/bin/gammaray.rs:5-112):

    let s = geom::Sphere::new(material::Material::disney().base_color(c).build(), xf, 5.0);
    let mut stage = render::Stage::new(prims);
    let mut film = render::Film::new(w, h);
    stage.trace(&camera, &render::PathTracerIntegrator {}, &mut film);

and here:

    s = Sphere(Material.disney().base_color(c).build(), xf, 5.0)
    stage = Stage([s, ...])
    film = Film(w, h)
    stage.trace(camera, PathTracerIntegrator(), film)

Each class cites the Rust item it mirrors.  Everything runs in the CUDA library
(`gammaray_gb300.load()`); passing `lib=` selects another implementation of the same
ABI, which is how the tests drive the CPU oracle.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field, replace

import numpy as np

from . import _abi
from ._abi import fptr, uptr

# ------------------------------------------------------------------ core


@dataclass(frozen=True)
class Quat:
    """core/quat.rs:4-17 — {real, imaginary}."""

    real: float = 1.0
    imaginary: tuple = (0.0, 0.0, 0.0)

    @staticmethod
    def identity() -> "Quat":
        return Quat()

    @staticmethod
    def axis_angle(axis, angle: float) -> "Quat":
        a = np.asarray(axis, dtype=np.float64)
        a = a / np.linalg.norm(a)
        s = math.sin(0.5 * angle)
        return Quat(math.cos(0.5 * angle), tuple(float(x) for x in a * s))


class Mat:
    """core/matrix.rs: 4x4, row-major, row-vector convention (v' = v * M)."""

    def __init__(self, m=None):
        self.m = np.eye(4, dtype=np.float32) if m is None else np.asarray(m, dtype=np.float32).reshape(4, 4)

    @staticmethod
    def identity() -> "Mat":
        return Mat()

    @staticmethod
    def translation(t) -> "Mat":  # matrix.rs:73-95
        m = np.eye(4, dtype=np.float32)
        m[3, :3] = np.asarray(t, dtype=np.float32)
        return Mat(m)

    @staticmethod
    def scale(k: float) -> "Mat":  # matrix.rs:51-71
        m = np.eye(4, dtype=np.float32)
        m[0, 0] = m[1, 1] = m[2, 2] = k
        return Mat(m)

    @staticmethod
    def rotation(q: Quat) -> "Mat":  # matrix.rs:97-121
        r = np.float32(q.real)
        x, y, z = (np.float32(v) for v in q.imaginary)
        two = np.float32(2.0)
        one = np.float32(1.0)
        m = np.eye(4, dtype=np.float32)
        m[0, 0] = one - two * (y * y + z * z)
        m[0, 1] = two * (x * y + z * r)
        m[0, 2] = two * (z * x - y * r)
        m[1, 0] = two * (x * y - z * r)
        m[1, 1] = one - two * (z * z + x * x)
        m[1, 2] = two * (y * z + x * r)
        m[2, 0] = two * (z * x + y * r)
        m[2, 1] = two * (y * z - x * r)
        m[2, 2] = one - two * (y * y + x * x)
        return Mat(m)

    def __matmul__(self, other: "Mat") -> "Mat":
        return Mat(self.m @ other.m)

    __mul__ = __matmul__

    def transform_points(self, p: np.ndarray) -> np.ndarray:  # xform.rs:41-47
        p = np.asarray(p, dtype=np.float32).reshape(-1, 3)
        h = np.concatenate([p, np.ones((len(p), 1), np.float32)], axis=1) @ self.m
        return (h[:, :3] / h[:, 3:4]).astype(np.float32)

    def transform_normals(self, n: np.ndarray) -> np.ndarray:  # xform.rs:56-61 (inverse transpose)
        inv = np.linalg.inv(self.m.astype(np.float64)).astype(np.float32)
        n = np.asarray(n, dtype=np.float32).reshape(-1, 3)
        return (n @ inv[:3, :3].T).astype(np.float32)


HORIZONTAL_APERTURE_35MM = 2.2  # core/camera.rs:8-9
VERTICAL_APERTURE_35MM = 1.6


@dataclass
class Camera:
    """core/camera.rs:12-61 — Camera::new(focal_length, h_ap, v_ap, f_stop, rotate, translate)."""

    focal_length: float = 5.0
    horizontal_aperture: float = HORIZONTAL_APERTURE_35MM
    vertical_aperture: float = VERTICAL_APERTURE_35MM
    f_stop: float = 8.0
    rotate: Quat = field(default_factory=Quat)
    translate: tuple = (0.0, 0.0, 0.0)

    @staticmethod
    def default() -> "Camera":  # camera.rs:37-40
        return Camera()

    @staticmethod
    def with_fov(fov_y_degrees: float, aspect: float = 1.0, rotate: Quat | None = None, translate=(0, 0, 0)):
        """Pinhole camera whose vertical field of view is `fov_y_degrees`:
        window_max().1 = v_ap / (2 f) = tan(fov/2) (camera.rs:76-79)."""
        v_ap = 1.0
        f = v_ap / (2.0 * math.tan(math.radians(fov_y_degrees) * 0.5))
        return Camera(f, v_ap * aspect, v_ap, 8.0, rotate or Quat(), tuple(translate))

    def aspect_ratio(self) -> float:
        return self.horizontal_aperture / self.vertical_aperture

    def desc(self) -> _abi.CameraDesc:
        d = _abi.CameraDesc()
        d.focal_length = self.focal_length
        d.horizontal_aperture = self.horizontal_aperture
        d.vertical_aperture = self.vertical_aperture
        d.f_stop = self.f_stop
        d.rotate[:] = [self.rotate.real, *self.rotate.imaginary]
        d.translate[:] = list(self.translate)
        return d


# -------------------------------------------------------------- material


class Material:
    """material/material.rs:20-59 — constructors of the closed material set."""

    def __init__(self, desc: _abi.MaterialDesc):
        self.desc = desc

    @staticmethod
    def diffuse_light(incandescence) -> "Material":
        d = _abi.MaterialDesc()
        d.kind = _abi.MATERIAL_DIFFUSE_LIGHT
        d.incandescence[:] = [float(x) for x in incandescence]
        d.base_color[:] = [float(x) for x in incandescence]
        return Material(d)

    @staticmethod
    def diffuse() -> "Material":
        d = _abi.MaterialDesc()
        d.kind = _abi.MATERIAL_DIFFUSE
        return Material(d)

    @staticmethod
    def mirror() -> "Material":
        d = _abi.MaterialDesc()
        d.kind = _abi.MATERIAL_MIRROR
        return Material(d)

    @staticmethod
    def disney() -> "DisneyMaterialBuilder":
        return DisneyMaterialBuilder()

    def has_light(self) -> bool:
        return self.desc.kind == _abi.MATERIAL_DIFFUSE_LIGHT


class DisneyMaterialBuilder:
    """material/material.rs:256-389 — chained setters, then build()."""

    _FIELDS = (
        "roughness",
        "anisotropic",
        "ior",
        "metallic",
        "specular_trans",
        "specular_tint",
        "sheen",
        "sheen_tint",
        "clearcoat",
        "clearcoat_gloss",
    )

    def __init__(self):
        # Defaults of DisneyMaterialBuilder::new (material.rs:276-290).
        self.values = dict(
            base_color=(1.0, 1.0, 1.0),
            roughness=0.5,
            anisotropic=0.0,
            ior=1.5,
            metallic=0.0,
            specular_trans=0.0,
            specular_tint=0.0,
            sheen=0.0,
            sheen_tint=0.5,
            clearcoat=0.0,
            clearcoat_gloss=0.1,
        )

    def base_color(self, c):
        self.values["base_color"] = tuple(float(x) for x in c)
        return self

    def __getattr__(self, name):
        if name in DisneyMaterialBuilder._FIELDS:

            def setter(v):
                self.values[name] = float(v)
                return self

            return setter
        raise AttributeError(name)

    def build(self) -> Material:
        d = _abi.MaterialDesc()
        d.kind = _abi.MATERIAL_DISNEY
        d.base_color[:] = list(self.values["base_color"])
        for k in DisneyMaterialBuilder._FIELDS:
            setattr(d, k, self.values[k])
        return Material(d)


# ----------------------------------------------------------------- geom


class Mesh:
    """geom/mesh.rs:50-188 — a triangle mesh in world space.

    `vertices` (V,3), `triangles` (T,3); optional per-triangle `tri_normals` (T,3)
    into `normals`, and `tri_uvs` into `uvs` (U,2).  `xf` is applied like
    Mesh::from_obj does: points by Xform::transform, normals by the inverse
    transpose and then normalised unless nearly zero (mesh.rs:101-117).
    """

    def __init__(self, material: Material, xf: Mat | None, vertices, triangles, normals=None, tri_normals=None,
                 uvs=None, tri_uvs=None):
        self.material = material
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        self.vertices = xf.transform_points(v) if xf is not None else v
        self.triangles = np.ascontiguousarray(triangles, dtype=np.uint32).reshape(-1, 3)
        self.normals = None
        self.tri_normals = None
        if normals is not None and tri_normals is not None:
            n = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
            if xf is not None:
                nn = xf.transform_normals(n)
                mag2 = (n * n).sum(axis=1)
                with np.errstate(divide="ignore", invalid="ignore"):  # nearly-zero rows are kept raw
                    unit = nn / np.sqrt((nn * nn).sum(axis=1, keepdims=True))
                n = np.where((mag2 < np.finfo(np.float32).eps)[:, None], n, unit).astype(np.float32)
            self.normals = np.ascontiguousarray(n)
            self.tri_normals = np.ascontiguousarray(tri_normals, dtype=np.uint32).reshape(-1, 3)
        self.uvs = None if uvs is None else np.ascontiguousarray(uvs, dtype=np.float32).reshape(-1, 2)
        self.tri_uvs = None if tri_uvs is None else np.ascontiguousarray(tri_uvs, dtype=np.uint32).reshape(-1, 3)

    @staticmethod
    def from_obj(material: Material, xf: Mat | None, path: str) -> "Mesh":
        from .obj import load_obj

        return load_obj(material, xf, path)

    def num_components(self) -> int:
        return len(self.triangles)

    def fill(self, d: _abi.PrimDesc, material_index: int):
        d.kind = _abi.PRIM_MESH
        d.material = material_index
        d.vertices = fptr(self.vertices)
        d.num_vertices = len(self.vertices)
        d.tri_vertices = uptr(self.triangles)
        d.num_tris = len(self.triangles)
        if self.normals is not None:
            d.normals = fptr(self.normals)
            d.num_normals = len(self.normals)
            d.tri_normals = uptr(self.tri_normals)
        if self.uvs is not None:
            d.uvs = fptr(self.uvs)
            d.num_uvs = len(self.uvs)
            d.tri_uvs = uptr(self.tri_uvs)


class Sphere:
    """geom/sphere.rs:9-24 — Sphere::new(material, xf_mat, radius); only the
    transformed origin is kept."""

    def __init__(self, material: Material, xf: Mat | None, radius: float):
        self.material = material
        self.radius = float(radius)
        origin = np.zeros((1, 3), np.float32)
        self.center = (xf.transform_points(origin)[0] if xf is not None else origin[0]).astype(np.float32)

    def num_components(self) -> int:
        return 1

    def fill(self, d: _abi.PrimDesc, material_index: int):
        d.kind = _abi.PRIM_SPHERE
        d.material = material_index
        d.center[:] = [float(x) for x in self.center]
        d.radius = self.radius


# --------------------------------------------------------------- render


@dataclass
class PathTracerIntegrator:
    """render/integrators.rs:39-100.  Defaults are the reference constants."""

    max_depth: int = 0
    rr_depth: int = 10
    rr_aggressive_depth: int = 20
    kind: int = _abi.INTEGRATOR_PATH_TRACER

    def params(self, lib: _abi.Lib) -> _abi.RenderParams:
        p = _abi.RenderParams()
        lib.gr_render_params_default(self.kind, C.byref(p))
        p.max_depth, p.rr_depth, p.rr_aggressive_depth = self.max_depth, self.rr_depth, self.rr_aggressive_depth
        return p


@dataclass
class BdptIntegrator:
    """render/integrators.rs:102-418 (BDPT_MAX_DEPTH = 16, roulette from length 4).

    Extensions, off by default: mis = 1 weights the strategies by the power heuristic;
    light_tracing = 1 adds the light-walk-to-camera strategy, splatted into the film."""

    max_depth: int = 16
    rr_depth: int = 4
    mis: int = 0
    light_tracing: int = 0
    kind: int = _abi.INTEGRATOR_BDPT

    def params(self, lib: _abi.Lib) -> _abi.RenderParams:
        p = _abi.RenderParams()
        lib.gr_render_params_default(self.kind, C.byref(p))
        p.max_depth, p.rr_depth, p.mis, p.light_tracing = self.max_depth, self.rr_depth, self.mis, self.light_tracing
        return p


@dataclass
class DisplayColorIntegrator:
    """render/integrators.rs:18-34."""

    kind: int = _abi.INTEGRATOR_DISPLAY_COLOR

    def params(self, lib: _abi.Lib) -> _abi.RenderParams:
        p = _abi.RenderParams()
        lib.gr_render_params_default(self.kind, C.byref(p))
        return p


def _default_lib(lib):
    if lib is not None:
        return lib
    from . import load

    return load()


class Film:
    """render/film.rs:38-53 — Film::new(width, height); `pixels` reads accum/weight back."""

    def __init__(self, width: int, height: int, lib: _abi.Lib | None = None):
        self.lib = _default_lib(lib)
        self.width, self.height = int(width), int(height)
        h = C.c_void_p()
        self.lib.call("gr_film_create", self.width, self.height, C.byref(h))
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.gr_film_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clear(self):
        self.lib.call("gr_film_clear", self.handle)

    def read(self):
        """(accum (H,W,3), weight (H,W)) as float32 — Film::pixels."""
        acc = np.empty((self.height, self.width, 3), np.float32)
        w = np.empty((self.height, self.width), np.float32)
        self.lib.call("gr_film_read", self.handle, fptr(acc), fptr(w))
        return acc, w

    @property
    def pixels(self):
        return self.read()

    def resolve(self) -> np.ndarray:
        rgb = np.empty((self.height, self.width, 3), np.float32)
        self.lib.call("gr_film_resolve", self.handle, fptr(rgb))
        return rgb

    def write_exr(self, path: str):
        """ExrWriter::update + write (render/exr.rs:168-199)."""
        self.lib.call("gr_film_write_exr", self.handle, str(path).encode())

    def passes(self) -> int:
        n = C.c_uint32()
        self.lib.call("gr_film_passes", self.handle, C.byref(n))
        return n.value

    def read_splat(self) -> np.ndarray:
        """Light-tracing splat sums (H,W,3) — the BDPT extension's splat buffer; resolve()
        adds them divided by passes()."""
        sp = np.empty((self.height, self.width, 3), np.float32)
        self.lib.call("gr_film_read_splat", self.handle, fptr(sp))
        return sp


def scene_desc(prims, environment=(0.0, 0.0, 0.0), bvh_width: int = 0, leaf_size: int = 0, build: int = 0):
    """gr_scene_desc for `prims` (materials deduplicated by identity, in first-use order).
    Returns (desc, keepalive); the keepalive owns the arrays the desc points into."""
    materials: list[Material] = []
    index = {}
    prim_descs = (_abi.PrimDesc * max(1, len(prims)))()
    for i, p in enumerate(prims):
        key = id(p.material)
        if key not in index:
            index[key] = len(materials)
            materials.append(p.material)
        p.fill(prim_descs[i], index[key])
    mat_descs = (_abi.MaterialDesc * max(1, len(materials)))(*[m.desc for m in materials])
    d = _abi.SceneDesc()
    d.materials = mat_descs
    d.num_materials = len(materials)
    d.prims = prim_descs
    d.num_prims = len(prims)
    d.environment[:] = [float(x) for x in environment]
    d.bvh_width = bvh_width
    d.leaf_size = leaf_size
    d.build = build
    return d, (materials, mat_descs, prim_descs, list(prims))


def plan_scene(prims, lib: _abi.Lib | None = None, environment=(0.0, 0.0, 0.0), bvh_width: int = 0,
               leaf_size: int = 0) -> _abi.SceneInfo:
    """gr_scene_plan: the BVH build and device footprint of a scene, on the host only."""
    lib = _default_lib(lib)
    d, keep = scene_desc(prims, environment, bvh_width, leaf_size)
    info = _abi.SceneInfo()
    lib.call("gr_scene_plan", C.byref(d), C.byref(info))
    return info


class Stage:
    """render/stage.rs:10-36 — owns the prims and their BVH; trace() renders one pass.

    Extensions (defaults reproduce the reference): `environment` radiance for escaped
    rays, device `bvh_width` / `leaf_size`, the random `seed`, and `device_build=True`
    for a BVH built on the GPU (GR_BUILD_DEVICE_LBVH) instead of the reference's host
    SAH build.
    """

    def __init__(self, prims, lib: _abi.Lib | None = None, environment=(0.0, 0.0, 0.0), bvh_width: int = 0,
                 leaf_size: int = 0, seed: int = 0, device_build: bool = False):
        self.lib = _default_lib(lib)
        self.prims = list(prims)
        self.seed = int(seed)
        self._pass = 0
        d, keep = scene_desc(self.prims, environment, bvh_width, leaf_size,
                             _abi.BUILD_DEVICE_LBVH if device_build else _abi.BUILD_HOST_SAH)
        h = C.c_void_p()
        self.lib.call("gr_scene_create", C.byref(d), C.byref(h))
        self.handle = h
        self.materials = keep[0]

    def close(self):
        if self.handle:
            self.lib.gr_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> _abi.SceneInfo:
        i = _abi.SceneInfo()
        self.lib.call("gr_scene_get_info", self.handle, C.byref(i))
        return i

    def last_stats(self) -> _abi.RenderStats:
        s = _abi.RenderStats()
        self.lib.call("gr_scene_last_stats", self.handle, C.byref(s))
        return s

    def params(self, integrator, spp: int = 1, first_pass: int | None = None) -> _abi.RenderParams:
        p = integrator.params(self.lib)
        p.spp = spp
        p.seed = self.seed
        p.first_pass = self._pass if first_pass is None else first_pass
        return p

    def trace(self, camera: Camera, integrator, film: Film):
        """Stage::trace (stage.rs:23-36): one jittered 1-spp pass splatted into `film`."""
        self.render(camera, integrator, film, spp=1)

    def render(self, camera: Camera, integrator, film: Film, spp: int):
        """`spp` consecutive trace() calls, in one library call."""
        p = self.params(integrator, spp)
        cam = camera.desc()
        self.lib.call("gr_render", self.handle, C.byref(cam), C.byref(p), film.handle)
        self._pass += spp

    def samples(self, camera: Camera, integrator, width: int, height: int, pass_index: int = 0) -> np.ndarray:
        """The FilmSample array of one pass: (H, W, 5) = s, t, r, g, b."""
        p = self.params(integrator, 1, pass_index)
        out = np.empty((height, width, 5), np.float32)
        cam = camera.desc()
        self.lib.call("gr_render_samples", self.handle, C.byref(cam), C.byref(p), width, height, fptr(out))
        return out

    # ---- ray queries (Bvh::intersect / intersect_naive / visibility / sample_light)
    def intersect(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        hits = np.zeros(len(rays), _abi.HIT_DTYPE)
        self.lib.call("gr_trace_rays", self.handle, fptr(rays), len(rays),
                      hits.ctypes.data_as(C.POINTER(_abi.Hit)))
        return hits

    def intersect_naive(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        hits = np.zeros(len(rays), _abi.HIT_DTYPE)
        self.lib.call("gr_intersect_naive", self.handle, fptr(rays), len(rays),
                      hits.ctypes.data_as(C.POINTER(_abi.Hit)))
        return hits

    def visibility(self, pairs: np.ndarray) -> np.ndarray:
        pairs = np.ascontiguousarray(pairs, dtype=np.float32).reshape(-1, 6)
        vis = np.zeros(len(pairs), np.uint8)
        self.lib.call("gr_visibility", self.handle, fptr(pairs), len(pairs),
                      vis.ctypes.data_as(C.POINTER(C.c_uint8)))
        return vis.astype(bool)

    def sample_light(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float32).reshape(-1, 6)
        out = np.zeros(len(u), _abi.LIGHT_SAMPLE_DTYPE)
        self.lib.call("gr_sample_light", self.handle, fptr(u), len(u),
                      out.ctypes.data_as(C.POINTER(_abi.LightSampleOut)))
        return out


# ------------------------------------------------------------ BSDF queries


def _frames(frames: np.ndarray):
    frames = np.ascontiguousarray(frames, dtype=_abi.FRAME_DTYPE)
    return frames, frames.ctypes.data_as(C.POINTER(_abi.Frame))


def bsdf_eval(material: Material, frames, wi, wo, camera_to_light=True, lib=None) -> np.ndarray:
    """Material::f_world for each row (material.rs:66-93)."""
    lib = _default_lib(lib)
    frames, fp = _frames(frames)
    wi = np.ascontiguousarray(wi, np.float32)
    wo = np.ascontiguousarray(wo, np.float32)
    f = np.empty((len(frames), 3), np.float32)
    lib.call("gr_bsdf_eval", C.byref(material.desc), len(frames), fp, fptr(wi), fptr(wo), int(camera_to_light),
             fptr(f))
    return f


def bsdf_pdf(material: Material, frames, wi, wo, lib=None) -> np.ndarray:
    """Material::pdf_world (material.rs:95-119)."""
    lib = _default_lib(lib)
    frames, fp = _frames(frames)
    wi = np.ascontiguousarray(wi, np.float32)
    wo = np.ascontiguousarray(wo, np.float32)
    p = np.empty(len(frames), np.float32)
    lib.call("gr_bsdf_pdf", C.byref(material.desc), len(frames), fp, fptr(wi), fptr(wo), fptr(p))
    return p


def bsdf_sample(material: Material, frames, wi, u, camera_to_light=True, lib=None) -> np.ndarray:
    """Material::sample_world with explicit uniforms (material.rs:140-235)."""
    lib = _default_lib(lib)
    frames, fp = _frames(frames)
    wi = np.ascontiguousarray(wi, np.float32)
    u = np.ascontiguousarray(u, np.float32)
    out = np.zeros(len(frames), _abi.BSDF_SAMPLE_DTYPE)
    lib.call("gr_bsdf_sample_batch", C.byref(material.desc), len(frames), fp, fptr(wi), fptr(u),
             int(camera_to_light), out.ctypes.data_as(C.POINTER(_abi.BsdfSample)))
    return out


def light_eval(material: Material, frames, wi, lib=None) -> np.ndarray:
    """Material::light_world (material.rs:123-134)."""
    lib = _default_lib(lib)
    frames, fp = _frames(frames)
    wi = np.ascontiguousarray(wi, np.float32)
    L = np.empty((len(frames), 3), np.float32)
    lib.call("gr_light_eval", C.byref(material.desc), len(frames), fp, fptr(wi), fptr(L))
    return L
