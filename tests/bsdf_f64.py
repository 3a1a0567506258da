"""A float64 numpy restatement of the reference's Disney material, written independently
of the C++ oracle so that each checks the other (test infrastructure only).

It follows, as written and with their quirks:
  - material/material.rs:292-333   DisneyMaterialBuilder::build (which lobes, weights);
  - material/material.rs:66-119    Material::f_world (lobes gated by the geometric
                                   normal's side) and Material::pdf_world (lobe average);
  - material/lobes.rs:93-116       DisneyDiffuseRefl (diffuse, retro-reflection, sheen);
  - material/lobes.rs:132-189      StandardMicrofacetRefl (specular and clearcoat);
  - material/lobes.rs:271-349      DisneySpecularTrans f and pdf;
  - material/lobes.rs:401-414      PerfectDiffuse; the default cosine pdf (lobes.rs:45-52);
  - material/util.rs               Schlick / dielectric / Disney Fresnel, GGX, GTR1;
  - core/vector.rs:137-234         the trig helpers (z read as cos(theta) even for a
                                   vector that is not of unit length) and tint().
All arrays are (n, 3) float64 in the local frame unless a name says world.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

INV_PI = 1.0 / math.pi


def _dot(a, b):
    return (a * b).sum(-1)


def _normalise(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def trig(v):
    """cos2(theta), sin2(theta), cos(phi), sin(phi) as core/vector.rs:137-205."""
    cos2 = v[:, 2] * v[:, 2]
    sin2 = np.maximum(0.0, 1.0 - cos2)
    sin = np.sqrt(sin2)
    safe = np.where(sin == 0, 1.0, sin)
    cphi = np.where(sin == 0, 1.0, np.clip(v[:, 0] / safe, -1, 1))
    sphi = np.where(sin == 0, 0.0, np.clip(v[:, 1] / safe, -1, 1))
    return cos2, sin2, cphi, sphi


def tint(c):  # core/vector.rs:218-234
    lum = 0.21 * c[0] + 0.71 * c[1] + 0.08 * c[2]
    return np.asarray(c, np.float64) / lum if lum > 0 else np.ones(3)


def lerp(a, b, t):
    return a + t * (b - a)


def schlick_weight(c):  # util.rs:8-11
    x = np.clip(1.0 - c, 0.0, 1.0)
    return x ** 5


def fresnel_dielectric(cos_in, ior):  # util.rs:21-46
    entering = cos_in > 0
    eta_i = np.where(entering, 1.0, ior)
    eta_t = np.where(entering, ior, 1.0)
    c = np.clip(np.where(entering, cos_in, -cos_in), 0.0, 1.0)
    sin_t = eta_i / eta_t * np.sqrt(np.maximum(0.0, 1.0 - c * c))
    cos_t = np.sqrt(np.maximum(0.0, 1.0 - sin_t * sin_t))
    with np.errstate(divide="ignore", invalid="ignore"):
        r_parl = (eta_t * c - eta_i * cos_t) / (eta_t * c + eta_i * cos_t)
        r_perp = (eta_i * c - eta_t * cos_t) / (eta_i * c + eta_t * cos_t)
    return np.where(sin_t >= 1.0, 1.0, (r_parl * r_parl + r_perp * r_perp) / 2.0)


class Ggx:  # util.rs:127-251
    def __init__(self, roughness, anisotropic):
        aspect = math.sqrt(1.0 - anisotropic * 0.9)
        self.ax = max(0.001, roughness * roughness / aspect)
        self.ay = max(0.001, roughness * roughness * aspect)

    def lam(self, v):
        _, sin2, cphi, sphi = trig(v)
        with np.errstate(divide="ignore", invalid="ignore"):
            tan = np.abs(np.sqrt(sin2) / v[:, 2])
        fin = np.isfinite(tan)
        alpha = np.sqrt(cphi ** 2 * self.ax ** 2 + sphi ** 2 * self.ay ** 2)
        a2t2 = (alpha * np.where(fin, tan, 0.0)) ** 2
        return np.where(fin, (-1.0 + np.sqrt(1.0 + a2t2)) * 0.5, 0.0)

    def g1(self, v):
        return 1.0 / (1.0 + self.lam(v))

    def d(self, h):
        cos2, sin2, cphi, sphi = trig(h)
        with np.errstate(divide="ignore", invalid="ignore"):
            tan2 = sin2 / cos2
            e = (cphi ** 2 / self.ax ** 2 + sphi ** 2 / self.ay ** 2) * tan2
            d = 1.0 / (math.pi * self.ax * self.ay * cos2 * cos2 * (1.0 + e) ** 2)
        return np.where(np.isfinite(tan2), d, 0.0)

    def g(self, i, o):
        return 1.0 / (1.0 + self.lam(i) + self.lam(o))

    def pdf(self, i, h):
        with np.errstate(divide="ignore", invalid="ignore"):
            p = self.d(h) * self.g1(i) * np.abs(_dot(i, h)) / np.abs(i[:, 2])
        return np.where(i[:, 2] == 0, 0.0, p)


class Gtr1:  # util.rs:256-309; lambda is written as the reference has it
    def __init__(self, gloss):
        self.alpha = lerp(0.1, 0.001, gloss)

    def lam(self, v):
        c = np.abs(v[:, 2])
        a2 = 0.25 * 0.25
        return 1.0 / (c + np.sqrt(a2 + c * c - a2 * c * c))

    def d(self, h):
        a2 = self.alpha * self.alpha
        c = np.abs(h[:, 2])
        return (a2 - 1.0) / (math.pi * math.log(a2) * (1.0 + (a2 - 1.0) * c * c))

    def g(self, i, o):
        return 1.0 / (1.0 + self.lam(i) + self.lam(o))

    def pdf(self, i, h):
        return self.d(h)


REFLECTION, TRANSMISSION = 1, 2


class DiffuseRefl:  # lobes.rs:75-116
    kind = REFLECTION

    def __init__(self, color, roughness, sheen, sheen_tint, weight):
        self.color = np.asarray(color, np.float64) * weight
        self.sheen = (sheen * weight) * lerp(np.ones(3), tint(color), sheen_tint)
        self.roughness = roughness

    def f(self, i, o, camera_to_light):
        f_in, f_out = schlick_weight(np.abs(i[:, 2])), schlick_weight(np.abs(o[:, 2]))
        diffuse = self.color * (INV_PI * (1 - 0.5 * f_in) * (1 - 0.5 * f_out))[:, None]
        hu = i + o
        zero = (hu == 0).all(-1)
        h = _normalise(np.where(zero[:, None], 1.0, hu))
        cd = _dot(o, h)
        rr = 2.0 * self.roughness * cd * cd
        retro = self.color * (INV_PI * rr * (f_out + f_in + f_out * f_in * (rr - 1.0)))[:, None]
        sheen = self.sheen * schlick_weight(cd)[:, None]
        return np.where(zero[:, None], diffuse, diffuse + (retro + sheen))

    def pdf(self, i, o):
        return np.where(i[:, 2] * o[:, 2] > 0, np.abs(o[:, 2]) * INV_PI, 0.0)


class PerfectDiffuse(DiffuseRefl):  # lobes.rs:401-414
    def __init__(self):
        pass

    def f(self, i, o, camera_to_light):
        return np.full((len(i), 3), 0.5 * INV_PI)


class MicrofacetRefl:  # lobes.rs:125-189
    kind = REFLECTION

    def __init__(self, dist, fresnel, color):
        self.dist, self.fresnel, self.color = dist, fresnel, np.asarray(color, np.float64)

    def f(self, i, o, camera_to_light):
        ci, co = np.abs(i[:, 2]), np.abs(o[:, 2])
        hu = i + o
        zero = (hu == 0).all(-1) | (ci == 0) | (co == 0)
        h = _normalise(np.where(zero[:, None], 1.0, hu))
        fr = self.fresnel(_dot(o, h))
        with np.errstate(divide="ignore", invalid="ignore"):
            s = self.dist.d(h) * self.dist.g(i, o) / (4.0 * co * ci)
        return np.where(zero[:, None], 0.0, self.color * fr * s[:, None])

    def pdf(self, i, o):
        same = i[:, 2] * o[:, 2] > 0
        h = _normalise(np.where(same[:, None], i + o, 1.0))
        with np.errstate(divide="ignore", invalid="ignore"):
            p = self.dist.pdf(i, h) / (4.0 * _dot(i, h))
        return np.where(same, p, 0.0)


def disney_fresnel(ior, color, specular_tint, metallic):  # util.rs:58-84
    color = np.asarray(color, np.float64)
    spec = lerp(np.ones(3), tint(color), specular_tint)

    def fr(c):
        dielectric = spec * fresnel_dielectric(c, ior)[:, None]
        conductor = lerp(color, np.ones(3), schlick_weight(c)[:, None])
        return lerp(dielectric, conductor, metallic)
    return fr


def schlick_fresnel(r0):  # util.rs:104-118
    return lambda c: lerp(np.full(3, r0), np.ones(3), schlick_weight(c)[:, None])


class SpecularTrans:  # lobes.rs:245-393
    kind = TRANSMISSION

    def __init__(self, color, roughness, anisotropic, ior):
        self.dist = Ggx(roughness, anisotropic)
        self.ior = max(ior, 1.01)
        self.color = np.asarray(color, np.float64)

    def _half(self, i, o, as_reference_pdf):
        eta = np.where(i[:, 2] > 0, self.ior, 1.0 / self.ior)
        hu = i + o * eta[:, None]
        hn = _normalise(hu)
        up = hu[:, 2:3] > 0
        h = np.where(up, hu if as_reference_pdf else hn, -hn)
        return eta, h

    def f(self, i, o, camera_to_light):
        ci, co = i[:, 2], o[:, 2]
        zero = (ci * co > 0) | (ci == 0) | (co == 0)
        eta, h = self._half(i, o, False)
        fr = fresnel_dielectric(_dot(o, h), self.ior)
        ih, oh = _dot(i, h), _dot(o, h)
        den = ih + eta * oh
        factor = 1.0 if camera_to_light else eta
        with np.errstate(divide="ignore", invalid="ignore"):
            s = np.abs(self.dist.d(h) * self.dist.g(i, o) * factor * factor * np.abs(oh) * np.abs(ih)
                       / (co * ci * den * den))
        return np.where(zero[:, None], 0.0, self.color * (1.0 - fr)[:, None] * s[:, None])

    def pdf(self, i, o, as_reference=True):
        """As lobes.rs:321-349 by default.  With as_reference=False, the density sample_f
        (lobes.rs:351-388) actually draws from: the half vector normalised and zero where
        the microfacet faces away from i or o."""
        eta, h = self._half(i, o, as_reference)
        ih, oh = _dot(i, h), _dot(o, h)
        den = ih + eta * oh
        with np.errstate(divide="ignore", invalid="ignore"):
            p = self.dist.pdf(i, h) * np.abs(eta * eta * oh / (den * den))
        zero = i[:, 2] * o[:, 2] > 0
        if not as_reference:
            zero |= (ih * i[:, 2] < 0) | (oh * o[:, 2] < 0)
        return np.where(zero, 0.0, p)


@dataclass
class Disney:
    """DisneyMaterialBuilder's parameters and defaults (material.rs:255-290)."""
    base_color: tuple = (1.0, 1.0, 1.0)
    roughness: float = 0.5
    anisotropic: float = 0.0
    ior: float = 1.5
    metallic: float = 0.0
    specular_trans: float = 0.0
    specular_tint: float = 0.0
    sheen: float = 0.0
    sheen_tint: float = 0.5
    clearcoat: float = 0.0
    clearcoat_gloss: float = 0.1

    def lobes(self):  # material.rs:292-333
        c = np.asarray(self.base_color, np.float64)
        dw = (1.0 - self.metallic) * (1.0 - self.specular_trans)
        tw = (1.0 - self.metallic) * self.specular_trans
        out = []
        if dw > 0:
            out.append(DiffuseRefl(c, self.roughness, self.sheen, self.sheen_tint, dw))
        if self.ior > 1.0:
            ior = max(self.ior, 1.01)
            out.append(MicrofacetRefl(Ggx(self.roughness, self.anisotropic),
                                      disney_fresnel(ior, c, self.specular_tint, self.metallic), np.ones(3)))
        if self.clearcoat > 0:
            out.append(MicrofacetRefl(Gtr1(self.clearcoat_gloss), schlick_fresnel(0.04),
                                      np.full(3, 0.25 * self.clearcoat)))
        if tw > 0:
            out.append(SpecularTrans(tw * np.sqrt(c), self.roughness, self.anisotropic, self.ior))
        return out

    def build(self, g):
        """The same material through the library's builder (`g` is gammaray_gb300)."""
        b = g.Material.disney().base_color(self.base_color)
        for k in ("roughness", "anisotropic", "ior", "metallic", "specular_trans", "specular_tint",
                  "sheen", "sheen_tint", "clearcoat", "clearcoat_gloss"):
            b = getattr(b, k)(getattr(self, k))
        return b.build()


def to_local(v, frames):  # core/vector.rs:112-116
    return np.stack([_dot(v, frames["tangent"].astype(np.float64)),
                     _dot(v, frames["binormal"].astype(np.float64)),
                     _dot(v, frames["normal"].astype(np.float64))], axis=-1)


def f_world(lobes, frames, wi, wo, camera_to_light=True):  # material.rs:66-93
    gn = frames["geom_normal"].astype(np.float64)
    reflect = _dot(wi, gn) * _dot(wo, gn) > 0
    i, o = to_local(wi, frames), to_local(wo, frames)
    out = np.zeros((len(wi), 3))
    for lobe in lobes:
        use = reflect if lobe.kind == REFLECTION else ~reflect
        out += np.where(use[:, None], lobe.f(i, o, camera_to_light), 0.0)
    return out


def pdf_world(lobes, frames, wi, wo):  # material.rs:95-119
    if not lobes:
        return np.zeros(len(wi))
    i, o = to_local(wi, frames), to_local(wo, frames)
    p = sum(lobe.pdf(i, o) for lobe in lobes) / len(lobes)
    return np.where(i[:, 2] == 0, 0.0, p)


# ------------------------------------------------------------------ sampling
def cosine_hemisphere(flipped, u1, u2):  # core/random.rs:28-56, 93-105
    sx, sy = -1.0 + 2.0 * u1, -1.0 + 2.0 * u2
    origin = (sx == 0) & (sy == 0)
    big_x = np.abs(sx) > np.abs(sy)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(big_x, sx, sy)
        theta = np.where(big_x, math.pi / 4 * (sy / sx), math.pi / 2 - math.pi / 4 * (sx / sy))
    x = np.where(origin, 0.0, r * np.cos(theta))
    y = np.where(origin, 0.0, r * np.sin(theta))
    z = np.sqrt(np.maximum(0.0, 1.0 - x * x - y * y))
    return np.stack([x, y, np.where(flipped, -z, z)], axis=-1)


def _ggx_sample11(cos_theta, u1, u2):  # util.rs:152-194
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.sqrt(u1 / (1.0 - u1))
        phi = 2.0 * math.pi * u2
        normal_x, normal_y = r * np.cos(phi), r * np.sin(phi)
        sin_t = np.sqrt(np.maximum(0.0, 1.0 - cos_theta * cos_theta))
        tan_t = sin_t / cos_theta
        g1 = 2.0 / (1.0 + np.sqrt(1.0 + tan_t * tan_t))
        a = 2.0 * u1 / g1 - 1.0
        tmp = np.minimum(1.0 / (a * a - 1.0), 1e10)
        b = tan_t
        d = np.sqrt(np.maximum(b * b * tmp * tmp - (a * a - b * b) * tmp, 0.0))
        sx1, sx2 = b * tmp - d, b * tmp + d
        slope_x = np.where((a < 0) | (sx2 > 1.0 / tan_t), sx1, sx2)
    s = np.where(u2 > 0.5, 1.0, -1.0)
    u = np.where(u2 > 0.5, 2.0 * (u2 - 0.5), 2.0 * (0.5 - u2))
    z = (u * (u * (u * 0.27385 - 0.73369) + 0.46341)) / (u * (u * (u * 0.093073 + 0.309420) - 1.000000) + 0.597999)
    slope_y = s * z * np.sqrt(1.0 + slope_x * slope_x)
    normal = cos_theta > 0.9999
    return np.where(normal, normal_x, slope_x), np.where(normal, normal_y, slope_y)


def ggx_sample_half(dist, i, u1, u2):  # util.rs:214-240
    flip = i[:, 2] < 0
    f = np.where(flip[:, None], -i, i)
    st = _normalise(np.stack([dist.ax * f[:, 0], dist.ay * f[:, 1], f[:, 2]], axis=-1))
    sx, sy = _ggx_sample11(st[:, 2], u1, u2)
    _, _, cphi, sphi = trig(st)
    rx = dist.ax * (cphi * sx - sphi * sy)
    ry = dist.ay * (sphi * sx + cphi * sy)
    h = _normalise(np.stack([-rx, -ry, np.ones_like(rx)], axis=-1))
    return np.where(flip[:, None], -h, h)


def gtr1_sample_half(dist, i, u1, u2):  # util.rs:282-298, precedence as written
    a2 = dist.alpha * dist.alpha
    phi = 2.0 * math.pi * u1
    c = np.sqrt(np.clip(1.0 - np.power(a2, 1.0 - u2) / (1.0 - a2), 0.0, 1.0))
    s = np.sqrt(1.0 - c * c)
    h = np.stack([s * np.cos(phi), s * np.sin(phi), c], axis=-1)
    return np.where((h[:, 2] * i[:, 2] > 0)[:, None], h, -h)


def reflect(v, n):  # core/vector.rs:240-246
    return n * (2.0 * _dot(n, v))[:, None] - v


def refract(v, n, eta):  # core/vector.rs:253-264
    c = _dot(n, v)
    s2t = eta * eta * np.maximum(0.0, 1.0 - c * c)
    ct = np.sqrt(np.maximum(0.0, 1.0 - s2t))
    o = -eta[:, None] * v + ((eta * c - ct)[:, None]) * n
    return np.where((s2t >= 1.0)[:, None], 0.0, o)


def lobe_sample(lobe, i, u1, u2, camera_to_light):
    """(result, outgoing, pdf) of Lobe::sample_f (lobes.rs:54-68, 160-184, 351-388)."""
    n = len(i)
    if isinstance(lobe, DiffuseRefl):
        o = cosine_hemisphere(i[:, 2] < 0, u1, u2)
        return lobe.f(i, o, camera_to_light), o, lobe.pdf(i, o)
    if isinstance(lobe, MicrofacetRefl):
        sample = ggx_sample_half if isinstance(lobe.dist, Ggx) else gtr1_sample_half
        h = sample(lobe.dist, i, u1, u2)
        o = reflect(i, h)
        ok = (i[:, 2] != 0) & (i[:, 2] * o[:, 2] > 0)
        with np.errstate(divide="ignore", invalid="ignore"):
            pdf = lobe.dist.pdf(i, h) / (4.0 * _dot(i, h))
        o = np.where(ok[:, None], o, 0.0)
        return np.where(ok[:, None], lobe.f(i, o, camera_to_light), 0.0), o, np.where(ok, pdf, 0.0)
    h = ggx_sample_half(lobe.dist, i, u1, u2)
    eta = np.where(i[:, 2] > 0, 1.0 / lobe.ior, lobe.ior)
    o = refract(i, h, eta)
    ok = (i[:, 2] != 0) & ~(o == 0).all(-1)
    o = np.where(ok[:, None], o, 0.0)
    res = np.where(ok[:, None], lobe.f(i, np.where(ok[:, None], o, 1.0), camera_to_light), 0.0)
    pdf = np.where(ok, lobe.pdf(i, np.where(ok[:, None], o, 1.0)), 0.0)
    return res, o, pdf


def lobe_index(u0, n):
    """Range::new(0, n) driven by one float32 uniform, as the library maps it."""
    r = (np.asarray(u0, np.float32) * np.float32(n)).astype(np.uint32)
    return np.minimum(r, n - 1)


def sample_world(lobes, frames, wi, u, camera_to_light=True):
    """(radiance, outgoing world, pdf, chosen lobe, valid) of Material::sample_world
    (material.rs:140-235) for a material without specular lobes: the pdf is the lobe
    average at the drawn direction, and the other lobes' values are added when the
    *chosen* lobe's kind matches the side of the geometric normal (material.rs:203-206)."""
    n = len(lobes)
    if n == 0:  # material.rs:166-174
        z = np.zeros((len(wi), 3))
        return z, z, np.ones(len(wi)), np.zeros(len(wi), np.uint32), np.zeros(len(wi), bool)
    i = to_local(wi, frames)
    r = lobe_index(u[:, 0], n)
    u1, u2 = u[:, 1].astype(np.float64), u[:, 2].astype(np.float64)
    res, o, pdf = np.zeros((len(i), 3)), np.zeros((len(i), 3)), np.zeros(len(i))
    for k, lobe in enumerate(lobes):
        rk, ok_, pk = lobe_sample(lobe, i, u1, u2, camera_to_light)
        sel = r == k
        res[sel], o[sel], pdf[sel] = rk[sel], ok_[sel], pk[sel]
    t, b, nn = (frames[f].astype(np.float64) for f in ("tangent", "binormal", "normal"))
    o_w = t * o[:, :1] + b * o[:, 1:2] + nn * o[:, 2:3]
    gn = frames["geom_normal"].astype(np.float64)
    reflect_side = _dot(wi, gn) * _dot(o_w, gn) > 0
    chosen_kind = np.array([lobes[k].kind for k in range(n)])[r]
    gate = (reflect_side & (chosen_kind == REFLECTION)) | (~reflect_side & (chosen_kind == TRANSMISSION))
    for k, lobe in enumerate(lobes):
        other = r != k
        pdf = pdf + np.where(other, lobe.pdf(i, o), 0.0)
        res = res + np.where((other & gate)[:, None], lobe.f(i, o, camera_to_light), 0.0)
    pdf = pdf / n
    valid = pdf != 0
    return np.where(valid[:, None], res, 0.0), o_w, np.where(valid, pdf, 1.0), r, valid
