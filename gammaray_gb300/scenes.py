"""Seeded synthetic scenes for the benchmark configurations.

The reference renders a hard-coded demo scene whose mesh asset is not distributed
(src/bin/gammaray.rs:5-58).  The workloads here are generated instead, from a seed:

  cornell_spheres   closed box of 5 walls (10 triangles, 2 m side), a 0.5 x 0.5 m
                    quad light of radiance 15 and two analytic spheres (r 0.3, 0.4);
                    Disney base 0.7 grey, roughness 0.5, metallic 0, ior 1.5.
                    256 x 256, 16 spp, max depth 8, roulette after depth 3.
  displaced_sphere  a 160 x 320 UV sphere (102,400 triangles) of radius 1, radially
                    displaced by 3-octave value noise of amplitude 0.1, on a
                    20-triangle ground plane, one quad light and a constant
                    environment of 0.2; per-object Disney parameters drawn from the
                    seed.  1024 x 1024, 64 spp, max depth 12 (path tracer), or BDPT at
                    512 x 512, 16 spp, max path length 10.
  batch_scenes      64 displaced spheres with log-uniform triangle counts in
                    [1k, 200k], 0-8 analytic spheres, random resolution, spp and depth.
  serving_scenes    16 resident displaced spheres with log-uniform counts in [10k, 2M].

All geometry is generated in world space as float32 arrays; the same arrays feed the
CUDA library and the CPU oracle.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .api import (
    BdptIntegrator,
    Camera,
    Material,
    Mesh,
    PathTracerIntegrator,
    Quat,
    Sphere,
)


@dataclass
class Workload:
    name: str
    prims: list
    camera: Camera
    integrator: object
    width: int
    height: int
    spp: int
    environment: tuple = (0.0, 0.0, 0.0)
    meta: dict = field(default_factory=dict)

    def num_triangles(self) -> int:
        return int(sum(p.num_components() for p in self.prims if isinstance(p, Mesh)))


# ----------------------------------------------------------------- geometry


def quad(corner, edge_u, edge_v):
    """Two triangles covering corner + [0,1] edge_u + [0,1] edge_v.  The geometric
    normal (a - c) x (b - c) of both triangles is edge_u x edge_v normalised
    (geom/mesh.rs:194-204)."""
    c = np.asarray(corner, np.float32)
    u = np.asarray(edge_u, np.float32)
    v = np.asarray(edge_v, np.float32)
    verts = np.stack([c, c + u, c + u + v, c + v]).astype(np.float32)
    # tri (a, b, c): (a - c) x (b - c) must equal +u x v.
    tris = np.array([[1, 2, 0], [2, 3, 0]], np.uint32)
    return verts, tris


def merge(parts):
    vs, ts, off = [], [], 0
    for v, t in parts:
        vs.append(v)
        ts.append(t + off)
        off += len(v)
    return np.concatenate(vs).astype(np.float32), np.concatenate(ts).astype(np.uint32)


def _lattice(ix, iy, iz, seed):
    h = (ix.astype(np.uint64) * np.uint64(0x8DA6B343)) ^ (iy.astype(np.uint64) * np.uint64(0xD8163841)) ^ (
        iz.astype(np.uint64) * np.uint64(0xCB1AB31F)) ^ np.uint64(seed * 0x9E3779B1 & 0xFFFFFFFF)
    h = h & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(16)
    h = (h * np.uint64(0x7FEB352D)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(15)
    h = (h * np.uint64(0x846CA68B)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(16)
    return (h.astype(np.float64) / 4294967295.0) * 2.0 - 1.0


def value_noise(p: np.ndarray, seed: int, octaves: int = 3) -> np.ndarray:
    """Sum of `octaves` octaves of trilinear value noise in [-1, 1] (frequency x2,
    amplitude /2 per octave), normalised by the total amplitude."""
    total = np.zeros(len(p))
    amp, freq, norm = 1.0, 2.0, 0.0
    for o in range(octaves):
        q = p * freq
        i = np.floor(q).astype(np.int64)
        f = q - i
        s = f * f * (3.0 - 2.0 * f)
        acc = np.zeros(len(p))
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    w = (s[:, 0] if dx else 1 - s[:, 0]) * (s[:, 1] if dy else 1 - s[:, 1]) * (
                        s[:, 2] if dz else 1 - s[:, 2])
                    acc += w * _lattice(i[:, 0] + dx + 1024, i[:, 1] + dy + 1024, i[:, 2] + dz + 1024, seed + 7 * o)
        total += amp * acc
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def displaced_uv_sphere(rings: int, segments: int, radius: float, amplitude: float, seed: int, center=(0, 0, 0)):
    """A rings x segments UV sphere (2 * rings * segments triangles, including the
    zero-area ones at the poles), radially displaced by value noise."""
    th = np.linspace(0.0, math.pi, rings + 1)
    ph = np.linspace(0.0, 2.0 * math.pi, segments + 1)
    T, P = np.meshgrid(th, ph, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(P), np.cos(T), np.sin(T) * np.sin(P)], axis=-1).reshape(-1, 3)
    r = radius * (1.0 + amplitude * value_noise(d * 1.5, seed))
    verts = (d * r[:, None] + np.asarray(center, np.float64)).astype(np.float32)
    idx = np.arange((rings + 1) * (segments + 1)).reshape(rings + 1, segments + 1)
    a = idx[:-1, :-1].ravel()
    b = idx[1:, :-1].ravel()
    c = idx[1:, 1:].ravel()
    dd = idx[:-1, 1:].ravel()
    tris = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, dd], 1)]).astype(np.uint32)
    return verts, tris


def ground_plane(y: float, half: float, nx: int = 2, nz: int = 5):
    """nx * nz quads (2 nx nz triangles) at height y, normal +y."""
    parts = []
    sx, sz = 2 * half / nx, 2 * half / nz
    for i in range(nx):
        for j in range(nz):
            corner = (-half + i * sx, y, -half + j * sz)
            parts.append(quad(corner, (0, 0, sz), (sx, 0, 0)))
    return merge(parts)


def random_disney(rng: np.random.Generator) -> Material:
    """baseColor U[.05,.95]^3, roughness U[.05,1], metallic ~ B(.3), clearcoat U[0,1],
    sheen U[0,1], specTrans ~ B(.2), ior 1.5."""
    b = Material.disney()
    b.base_color(rng.uniform(0.05, 0.95, 3))
    b.roughness(rng.uniform(0.05, 1.0))
    b.metallic(1.0 if rng.random() < 0.3 else 0.0)
    b.clearcoat(rng.uniform(0.0, 1.0))
    b.sheen(rng.uniform(0.0, 1.0))
    b.specular_trans(1.0 if rng.random() < 0.2 else 0.0)
    b.ior(1.5)
    return b.build()


# ------------------------------------------------------------------ scenes


def cornell_spheres(width=256, height=256, spp=16, seed=1) -> Workload:
    grey = Material.disney().base_color((0.7, 0.7, 0.7)).roughness(0.5).metallic(0.0).ior(1.5).build()
    walls = merge([
        quad((-1, 0, -1), (0, 0, 2), (2, 0, 0)),   # floor, normal +y
        quad((-1, 2, -1), (2, 0, 0), (0, 0, 2)),   # ceiling, normal -y
        quad((-1, 0, -1), (2, 0, 0), (0, 2, 0)),   # back wall, normal +z
        quad((-1, 0, -1), (0, 2, 0), (0, 0, 2)),   # left wall, normal +x
        quad((1, 0, -1), (0, 0, 2), (0, 2, 0)),    # right wall, normal -x
    ])
    lv, lt = quad((-0.25, 1.999, -0.25), (0.5, 0, 0), (0, 0, 0.5))  # normal -y: emits downwards
    light = Material.diffuse_light((15.0, 15.0, 15.0))
    prims = [
        Mesh(grey, None, *walls),
        Mesh(light, None, lv, lt),
        Sphere(grey, None, 0.3),
        Sphere(grey, None, 0.4),
    ]
    prims[2].center = np.array([-0.45, 0.3, -0.25], np.float32)
    prims[3].center = np.array([0.45, 0.4, 0.25], np.float32)
    cam = Camera.with_fov(40.0, width / height, translate=(0.0, 1.0, 3.7))
    integ = PathTracerIntegrator(max_depth=8, rr_depth=3, rr_aggressive_depth=20)
    return Workload("cornell_spheres", prims, cam, integ, width, height, spp, (0.0, 0.0, 0.0),
                    {"triangles": 12, "spheres": 2})


def _displaced_prims(rng, tris_target, seed, spheres=0):
    rings = max(4, int(round(math.sqrt(tris_target / 4.0))))
    segments = 2 * rings
    sv, st = displaced_uv_sphere(rings, segments, 1.0, 0.1, seed)
    gv, gt = ground_plane(-1.15, 6.0)
    lv, lt = quad((-0.5, 3.0, -0.5), (1.0, 0, 0), (0, 0, 1.0))
    prims = [
        Mesh(random_disney(rng), None, sv, st),
        Mesh(random_disney(rng), None, gv, gt),
        Mesh(Material.diffuse_light((10.0, 10.0, 10.0)), None, lv, lt),
    ]
    for k in range(spheres):
        r = float(rng.uniform(0.1, 0.35))
        ang = float(rng.uniform(0, 2 * math.pi))
        dist = float(rng.uniform(1.4, 2.6))
        s = Sphere(random_disney(rng), None, r)
        s.center = np.array([dist * math.cos(ang), -1.15 + r, dist * math.sin(ang)], np.float32)
        prims.append(s)
    return prims


def displaced_sphere(width=1024, height=1024, spp=64, seed=2, bdpt=False, tris=102_400) -> Workload:
    rng = np.random.default_rng(seed)
    rings = 160 if tris == 102_400 else None
    if rings:
        sv, st = displaced_uv_sphere(160, 320, 1.0, 0.1, seed)
        gv, gt = ground_plane(-1.15, 6.0)
        lv, lt = quad((-0.5, 3.0, -0.5), (1.0, 0, 0), (0, 0, 1.0))
        prims = [
            Mesh(random_disney(rng), None, sv, st),
            Mesh(random_disney(rng), None, gv, gt),
            Mesh(Material.diffuse_light((10.0, 10.0, 10.0)), None, lv, lt),
        ]
    else:
        prims = _displaced_prims(rng, tris, seed)
    cam = Camera.with_fov(40.0, width / height, translate=(0.0, 0.25, 4.6))
    if bdpt:
        integ = BdptIntegrator(max_depth=10, rr_depth=4)
        name = "bdpt_displaced_sphere"
    else:
        integ = PathTracerIntegrator(max_depth=12, rr_depth=10, rr_aggressive_depth=20)
        name = "pt_displaced_sphere"
    return Workload(name, prims, cam, integ, width, height, spp, (0.2, 0.2, 0.2),
                    {"triangles": int(sum(p.num_components() for p in prims if isinstance(p, Mesh)))})


def displaced_sphere_lobes(width=64, height=64, spp=1, bdpt=False) -> Workload:
    """The 102,400-triangle displaced sphere with its seeded materials (a rough glass
    sphere with clearcoat and sheen, a clearcoated ground with sheen), plus two analytic
    spheres so that every Disney lobe is on screen: a rough metal (roughness 0.3) and a
    rough dielectric with full sheen and a glossy clearcoat.  Both float 0.1 above the
    ground (a contact point would put connection vertices arbitrarily close together)."""
    w = displaced_sphere(width, height, spp, bdpt=bdpt)
    D = Material.disney
    metal = D().base_color((0.9, 0.6, 0.3)).metallic(1.0).roughness(0.3).build()
    coat = D().base_color((0.2, 0.5, 0.8)).roughness(0.6).sheen(1.0).clearcoat(1.0).clearcoat_gloss(0.8).build()
    s1, s2 = Sphere(metal, None, 0.4), Sphere(coat, None, 0.35)
    s1.center = np.array([-1.55, -0.65, 0.9], np.float32)
    s2.center = np.array([1.5, -0.7, 0.8], np.float32)
    w.prims = w.prims + [s1, s2]
    w.name += "_lobes"
    return w


def orbit_camera(rng, width, height, radius=4.6):
    """A random pose on a ring around the origin, looking at it.  The reference's
    camera origin is translate * rotation (core/camera.rs:50-52, row vectors), so the
    translation is pre-rotated by the inverse rotation."""
    yaw = float(rng.uniform(-math.pi, math.pi))
    q = Quat.axis_angle((0, 1, 0), yaw)
    pos = np.array([radius * math.sin(yaw), 0.25, radius * math.cos(yaw)])
    from .api import Mat

    R = Mat.rotation(q).m[:3, :3].astype(np.float64)
    t = pos @ np.linalg.inv(R)
    return Camera.with_fov(40.0, width / height, rotate=q, translate=tuple(float(x) for x in t))


def batch_scenes(n=64, seed=4):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        tris = int(math.exp(rng.uniform(math.log(1_000), math.log(200_000))))
        prims = _displaced_prims(rng, tris, seed * 1000 + k, spheres=int(rng.integers(0, 9)))
        res = [(128, 128), (256, 256), (512, 512), (1024, 576)][int(rng.integers(0, 4))]
        spp = int(rng.integers(4, 65))
        depth = int(rng.integers(4, 13))
        cam = orbit_camera(rng, *res)
        integ = PathTracerIntegrator(max_depth=depth, rr_depth=10, rr_aggressive_depth=20)
        out.append(Workload(f"batch{k}", prims, cam, integ, res[0], res[1], spp, (0.2, 0.2, 0.2),
                            {"triangles": tris}))
    return out


def serving_scenes(n=16, seed=5, max_tris=2_000_000):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        tris = int(math.exp(rng.uniform(math.log(10_000), math.log(max_tris))))
        prims = _displaced_prims(rng, tris, seed * 1000 + k, spheres=int(rng.integers(0, 9)))
        out.append((prims, (0.2, 0.2, 0.2)))
    return out
