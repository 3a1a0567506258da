// Device Disney BSDF: eval / pdf / sample for the lobe set of the reference
// (material/lobes.rs, material/util.rs) and the lobe mixture of Material
// (material/material.rs:66-235).  Every expression keeps the reference's operation
// order so results match it to a few ulp (the transcendental functions are CUDA's).
// Random draws arrive as explicit uniforms, in the order the reference draws them.
#pragma once

#include "common.cuh"

namespace gr {

// Lobe::f and Lobe::pdf are inlined; the sampling mixture calls each from one place
// only, to keep the shading kernels small enough for the instruction cache.
// GR_LOBE_CALLS builds them as real calls instead (measured slower).
#ifdef GR_LOBE_CALLS
#define GR_LOBE static __device__ __noinline__
#else
#define GR_LOBE GR_D
#endif

GR_D V3 ld3(const float* p) { return V3{p[0], p[1], p[2]}; }

// Local-frame trigonometry (core/vector.rs:137-213).
GR_D float cos2_theta(V3 v) { return v.z * v.z; }
GR_D float sin2_theta(V3 v) { return fmaxf(0.0f, 1.0f - cos2_theta(v)); }
GR_D float sin_theta(V3 v) { return sqrtf(sin2_theta(v)); }
GR_D float tan_theta(V3 v) { return sin_theta(v) / v.z; }
GR_D float tan2_theta(V3 v) { return sin2_theta(v) / cos2_theta(v); }
GR_D float cos_phi(V3 v) {
    float s = sin_theta(v);
    return s == 0.0f ? 1.0f : clampf(v.x / s, -1.0f, 1.0f);
}
GR_D float sin_phi(V3 v) {
    float s = sin_theta(v);
    return s == 0.0f ? 0.0f : clampf(v.y / s, -1.0f, 1.0f);
}
GR_D float cos2_phi(V3 v) { return cos_phi(v) * cos_phi(v); }
GR_D float sin2_phi(V3 v) { return sin_phi(v) * sin_phi(v); }
GR_D bool same_hemisphere(V3 a, V3 b) { return a.z * b.z > 0.0f; }

GR_D V3 reflect(V3 v, V3 n) {  // core/vector.rs:240-246
    float k = 2.0f * dot(n, v);
    return V3{n.x * k - v.x, n.y * k - v.y, n.z * k - v.z};
}
GR_D V3 refract(V3 v, V3 n, float eta) {  // core/vector.rs:253-264
    float ci = dot(n, v);
    float s2i = fmaxf(0.0f, 1.0f - ci * ci);
    float s2t = eta * eta * s2i;
    if (s2t >= 1.0f) return v3zero();
    float ct = sqrtf(1.0f - s2t);
    V3 a = V3{v.x * -eta, v.y * -eta, v.z * -eta};
    float k = eta * ci - ct;
    return V3{a.x + n.x * k, a.y + n.y * k, a.z + n.z * k};
}

// cosf and sinf of one angle.  Out of line so that the full-range argument reduction
// of both exists once in each shading kernel instead of at every sampler.
// Returns (cos a, sin a) by value, in registers.  GR_TRIG_INLINE inlines it instead.
#ifdef GR_TRIG_INLINE
GR_D float2 cos_sin(float a) { return make_float2(cosf(a), sinf(a)); }
#else
static __device__ __noinline__ float2 cos_sin(float a) { return make_float2(cosf(a), sinf(a)); }
#endif

// core/random.rs:28-106
GR_D void area_sample_disk(float u1, float u2, float& dx, float& dy) {
    float sx = -1.0f + 2.0f * u1;
    float sy = -1.0f + 2.0f * u2;
    if (sx == 0.0f && sy == 0.0f) {
        dx = 0.0f;
        dy = 0.0f;
        return;
    }
    float r, theta;
    if (fabsf(sx) > fabsf(sy)) {
        r = sx;
        theta = FRAC_PI_4 * (sy / sx);
    } else {
        r = sy;
        theta = FRAC_PI_2 - FRAC_PI_4 * (sx / sy);
    }
    float2 cs = cos_sin(theta);
    dx = r * cs.x;
    dy = r * cs.y;
}
GR_D V3 cosine_sample_hemisphere(bool flipped, float u1, float u2) {
    float x, y;
    area_sample_disk(u1, u2, x, y);
    float z = sqrtf(fmaxf(0.0f, 1.0f - x * x - y * y));
    return flipped ? V3{x, y, -1.0f * z} : V3{x, y, z};
}
GR_D float cosine_pdf(V3 d) { return fabsf(d.z) * FRAC_1_PI; }

// material/util.rs:8-49
GR_D float schlick_weight(float c) {
    float x = clamp_unit(1.0f - c);
    return x * x * x * x * x;
}
GR_D V3 fresnel_schlick(float c, V3 r0) { return vlerp(r0, v3one(), schlick_weight(c)); }
GR_D float fresnel_dielectric(float cos_in, float ior) {
    bool entering = cos_in > 0.0f;
    float ei, et, c;
    if (entering) {
        ei = 1.0f;
        et = ior;
        c = clamp_unit(cos_in);
    } else {
        ei = ior;
        et = 1.0f;
        c = clamp_unit(-cos_in);
    }
    float si = sqrtf(fmaxf(0.0f, 1.0f - c * c));
    float st = ei / et * si;
    if (st >= 1.0f) return 1.0f;
    float ct = sqrtf(fmaxf(0.0f, 1.0f - st * st));
    float rpl = ((et * c) - (ei * ct)) / ((et * c) + (ei * ct));
    float rpp = ((ei * c) - (et * ct)) / ((ei * c) + (et * ct));
    return (rpl * rpl + rpp * rpp) / 2.0f;
}

// ------------------------------------------------------------ GGX (util.rs:119-251)
GR_D float ggx_lambda(float ax, float ay, V3 v) {
    float att = fabsf(tan_theta(v));
    if (isfinite(att)) {
        float alpha = sqrtf(cos2_phi(v) * (ax * ax) + sin2_phi(v) * (ay * ay));
        float a2t2 = (alpha * att) * (alpha * att);
        return (-1.0f + sqrtf(1.0f + a2t2)) * 0.5f;
    }
    return 0.0f;
}
GR_D float ggx_g1(float ax, float ay, V3 v) { return 1.0f / (1.0f + ggx_lambda(ax, ay, v)); }
GR_D float ggx_g(float ax, float ay, V3 i, V3 o) {
    return 1.0f / (1.0f + ggx_lambda(ax, ay, i) + ggx_lambda(ax, ay, o));
}
GR_D float ggx_d(float ax, float ay, V3 h) {
    float t2 = tan2_theta(h);
    if (isfinite(t2)) {
        float c4 = cos2_theta(h) * cos2_theta(h);
        float e = (cos2_phi(h) / (ax * ax) + sin2_phi(h) / (ay * ay)) * t2;
        return 1.0f / (PI * ax * ay * c4 * (1.0f + e) * (1.0f + e));
    }
    return 0.0f;
}
GR_D float ggx_pdf(float ax, float ay, V3 i, V3 h) {
    float c = i.z;
    if (c == 0.0f) return 0.0f;
    return ggx_d(ax, ay, h) * ggx_g1(ax, ay, i) * fabsf(dot(i, h)) / fabsf(c);
}
GR_D void ggx_sample11(float cos_theta, float u1, float u2, float& sx, float& sy) {
    if (cos_theta > 0.9999f) {
        float r = sqrtf(u1 / (1.0f - u1));
        float phi = TWO_PI * u2;
        float2 cs = cos_sin(phi);
        sx = r * cs.x;
        sy = r * cs.y;
        return;
    }
    float s = sqrtf(fmaxf(0.0f, 1.0f - cos_theta * cos_theta));
    float t = s / cos_theta;
    float g1 = 2.0f / (1.0f + sqrtf(1.0f + t * t));
    float a = 2.0f * u1 / g1 - 1.0f;
    float tmp = fminf(1.0f / (a * a - 1.0f), 1e10f);
    float b = t;
    float d = sqrtf(fmaxf(b * b * tmp * tmp - (a * a - b * b) * tmp, 0.0f));
    float x1 = b * tmp - d;
    float x2 = b * tmp + d;
    float slope_x = (a < 0.0f || x2 > 1.0f / t) ? x1 : x2;
    float sg, u;
    if (u2 > 0.5f) {
        sg = 1.0f;
        u = 2.0f * (u2 - 0.5f);
    } else {
        sg = -1.0f;
        u = 2.0f * (0.5f - u2);
    }
    float z = (u * (u * (u * 0.27385f - 0.73369f) + 0.46341f)) /
              (u * (u * (u * 0.093073f + 0.309420f) - 1.000000f) + 0.597999f);
    sx = slope_x;
    sy = sg * z * sqrtf(1.0f + slope_x * slope_x);
}
GR_D V3 ggx_sample_half(float ax, float ay, V3 i, float u1, float u2) {
    bool flip = i.z < 0.0f;
    V3 f = flip ? -i : i;
    V3 st = normalized(V3{ax * f.x, ay * f.y, f.z});
    float sx, sy;
    ggx_sample11(st.z, u1, u2, sx, sy);
    float cp = cos_phi(st), sp = sin_phi(st);
    float xr = ax * (cp * sx - sp * sy);
    float yr = ay * (sp * sx + cp * sy);
    V3 h = normalized(V3{-xr, -yr, 1.0f});
    return flip ? -h : h;
}

// ----------------------------------------------------------- GTR1 (util.rs:255-309)
GR_D float gtr1_lambda(V3 v) {
    float ag = 0.25f;
    float c = fabsf(v.z);
    float a2 = ag * ag;
    float c2 = c * c;
    return 1.0f / (c + sqrtf(a2 + c2 - (a2 * c2)));
}
GR_D float gtr1_d(float alpha, V3 h) {
    float a2 = alpha * alpha;
    float c = fabsf(h.z);
    return (a2 - 1.0f) / (PI * logf(a2) * (1.0f + (a2 - 1.0f) * c * c));
}
GR_D float gtr1_g(V3 i, V3 o) { return 1.0f / (1.0f + gtr1_lambda(i) + gtr1_lambda(o)); }
GR_D V3 gtr1_sample_half(float alpha, V3 i, float u1, float u2) {
    float a2 = alpha * alpha;
    float phi = 2.0f * PI * u1;
    float c = sqrtf(clamp_unit(1.0f - powf(a2, 1.0f - u2) / (1.0f - a2)));
    float s = sqrtf(1.0f - c * c);  // Vec::from_spherical (core/vector.rs:21-24)
    float2 cs = cos_sin(phi);
    V3 h = V3{s * cs.x, s * cs.y, c};
    return same_hemisphere(h, i) ? h : -h;
}

// -------------------------------------------------------------- lobe dispatch
GR_D V3 microfacet_fresnel(const DevLobe& L, float c) {
    if (L.type == L_GGX_DISNEY) {  // DisneyFresnel (util.rs:72-78)
        V3 spec = ld3(L.c1);
        V3 dielectric = spec * fresnel_dielectric(c, L.p[2]);
        V3 conductor = fresnel_schlick(c, ld3(L.c0));
        return vlerp(dielectric, conductor, L.p[3]);
    }
    return fresnel_schlick(c, ld3(L.c1));  // SchlickFresnel (util.rs:106-110)
}
GR_D float microfacet_d(const DevLobe& L, V3 h) {
    return L.type == L_GGX_DISNEY ? ggx_d(L.p[0], L.p[1], h) : gtr1_d(L.p[0], h);
}
GR_D float microfacet_g(const DevLobe& L, V3 i, V3 o) {
    return L.type == L_GGX_DISNEY ? ggx_g(L.p[0], L.p[1], i, o) : gtr1_g(i, o);
}
GR_D float microfacet_pdf(const DevLobe& L, V3 i, V3 h) {
    return L.type == L_GGX_DISNEY ? ggx_pdf(L.p[0], L.p[1], i, h) : gtr1_d(L.p[0], h);
}

// Lobe::f
GR_LOBE V3 lobe_f(const DevLobe& L, V3 i, V3 o, bool c2l) {
    switch (L.type) {
        case L_DISNEY_DIFFUSE: {  // lobes.rs:93-116
            V3 color = ld3(L.c0);
            float fi = schlick_weight(fabsf(i.z));
            float fo = schlick_weight(fabsf(o.z));
            V3 diffuse = color * (FRAC_1_PI * (1.0f - 0.5f * fi) * (1.0f - 0.5f * fo));
            V3 hu = i + o;
            if (is_zero(hu)) return diffuse;
            V3 h = normalized(hu);
            float ctd = dot(o, h);
            float rr = 2.0f * L.p[0] * ctd * ctd;
            V3 retro = color * (FRAC_1_PI * rr * (fo + fi + fo * fi * (rr - 1.0f)));
            V3 sheen = ld3(L.c1) * schlick_weight(ctd);
            return diffuse + (retro + sheen);
        }
        case L_GGX_DISNEY:
        case L_GTR1_SCHLICK: {  // lobes.rs:135-148
            float ci = fabsf(i.z), co = fabsf(o.z);
            V3 hu = i + o;
            if (is_zero(hu) || ci == 0.0f || co == 0.0f) return v3zero();
            V3 h = normalized(hu);
            V3 fr = microfacet_fresnel(L, dot(o, h));
            float d = microfacet_d(L, h);
            float g = microfacet_g(L, i, o);
            V3 color = L.type == L_GGX_DISNEY ? v3one() : ld3(L.c0);
            return mul(color, fr) * (d * g / (4.0f * co * ci));
        }
        case L_SPECULAR_TRANS: {  // lobes.rs:272-319
            if (same_hemisphere(i, o)) return v3zero();
            float ci = i.z, co = o.z;
            if (ci == 0.0f || co == 0.0f) return v3zero();
            float ior = L.p[2];
            float eta = ci > 0.0f ? ior : 1.0f / ior;
            V3 hu = i + (o * eta);
            V3 h = hu.z > 0.0f ? normalized(hu) : -normalized(hu);
            float fr = fresnel_dielectric(dot(o, h), ior);
            V3 frv = v3one() * fr;
            float d = ggx_d(L.p[0], L.p[1], h);
            float g = ggx_g(L.p[0], L.p[1], i, o);
            float sd = dot(i, h) + eta * dot(o, h);
            float factor = c2l ? 1.0f : eta;
            V3 finv = v3one() - frv;
            return mul(ld3(L.c0), finv) *
                   fabsf(d * g * factor * factor * fabsf(dot(o, h)) * fabsf(dot(i, h)) / (co * ci * sd * sd));
        }
        case L_PERFECT_DIFFUSE:
            return V3{0.5f, 0.5f, 0.5f} * FRAC_1_PI;
        case L_PERFECT_MIRROR:
        default:
            return v3one() / fabsf(o.z);
    }
}

// Lobe::pdf
GR_LOBE float lobe_pdf(const DevLobe& L, V3 i, V3 o) {
    switch (L.type) {
        case L_GGX_DISNEY:
        case L_GTR1_SCHLICK: {  // lobes.rs:150-158
            if (!same_hemisphere(i, o)) return 0.0f;
            V3 h = normalized(i + o);
            return microfacet_pdf(L, i, h) / (4.0f * dot(i, h));
        }
        case L_SPECULAR_TRANS: {  // lobes.rs:321-349 (unnormalised half kept)
            if (same_hemisphere(i, o)) return 0.0f;
            float ior = L.p[2];
            float eta = i.z > 0.0f ? ior : 1.0f / ior;
            V3 hu = i + (o * eta);
            V3 h = hu.z > 0.0f ? hu : -normalized(hu);
            float sd = dot(i, h) + eta * dot(o, h);
            float dwh = fabsf((eta * eta * dot(o, h)) / (sd * sd));
            return ggx_pdf(L.p[0], L.p[1], i, h) * dwh;
        }
        case L_PERFECT_MIRROR:
            return 1.0f;
        default:  // lobes.rs:45-52
            if (!same_hemisphere(i, o)) return 0.0f;
            return cosine_pdf(o);
    }
}

// Lobe::sample_f, direction part.  Returns how the chosen lobe's value and pdf follow:
// SAMPLE_NONE (the sampler gave up: value, direction and pdf are zero), SAMPLE_PDF_GIVEN
// (microfacet reflection: the pdf is the sampler's, from the sampled half vector) or
// SAMPLE_PDF_EVAL (the pdf is Lobe::pdf of the sampled direction).  The value is always
// Lobe::f of the sampled direction, evaluated by the caller.
enum : int { SAMPLE_NONE = 0, SAMPLE_PDF_GIVEN = 1, SAMPLE_PDF_EVAL = 2 };

GR_D int lobe_direction(const DevLobe& L, V3 i, float u1, float u2, V3& o, float& pdf) {
    o = v3zero();
    pdf = 0.0f;
    switch (L.type) {
        case L_GGX_DISNEY:
        case L_GTR1_SCHLICK: {  // lobes.rs:160-184
            if (i.z == 0.0f) return SAMPLE_NONE;
            V3 h = L.type == L_GGX_DISNEY ? ggx_sample_half(L.p[0], L.p[1], i, u1, u2)
                                          : gtr1_sample_half(L.p[0], i, u1, u2);
            V3 r = reflect(i, h);
            if (!same_hemisphere(i, r)) return SAMPLE_NONE;
            o = r;
            pdf = microfacet_pdf(L, i, h) / (4.0f * dot(i, h));
            return SAMPLE_PDF_GIVEN;
        }
        case L_SPECULAR_TRANS: {  // lobes.rs:351-388
            if (i.z == 0.0f) return SAMPLE_NONE;
            V3 h = ggx_sample_half(L.p[0], L.p[1], i, u1, u2);
            float ior = L.p[2];
            float eta = i.z > 0.0f ? 1.0f / ior : ior;
            V3 r = refract(i, h, eta);
            if (is_zero(r)) return SAMPLE_NONE;
            o = r;
            return SAMPLE_PDF_EVAL;
        }
        case L_PERFECT_MIRROR:  // lobes.rs:440-452 (Lobe::pdf of a mirror is 1)
            o = V3{-i.x, -i.y, i.z};
            return SAMPLE_PDF_EVAL;
        default:  // lobes.rs:54-68
            o = cosine_sample_hemisphere(i.z < 0.0f, u1, u2);
            return SAMPLE_PDF_EVAL;
    }
}

// ------------------------------------------------------------ material mixture
GR_D V3 light_world(const DevMaterial& m, V3 wi, const Frame& f) {  // material.rs:123-134, lights.rs:15-21
    if (m.has_light && dot(wi, f.geom_normal) > 0.0f) return ld3(m.emission);
    return v3zero();
}

GR_D V3 f_world(const DevMaterial& m, V3 wi, V3 wo, const Frame& f, bool c2l) {  // material.rs:66-93
    V3 il = world_to_local(wi, f.tangent, f.binormal, f.normal);
    V3 ol = world_to_local(wo, f.tangent, f.binormal, f.normal);
    bool refl = (dot(wi, f.geom_normal) * dot(wo, f.geom_normal)) > 0.0f;
    V3 r = v3zero();
#pragma unroll 1
    for (int k = 0; k < m.n_lobes; ++k) {
        uint32_t kind = m.lobe[k].kind;
        if ((refl && (kind & LOBE_REFLECTION)) || (!refl && (kind & LOBE_TRANSMISSION)))
            r = r + lobe_f(m.lobe[k], il, ol, c2l);
    }
    return r;
}

GR_D float pdf_world(const DevMaterial& m, V3 wi, V3 wo, const Frame& f) {  // material.rs:95-119
    if (m.n_lobes == 0) return 0.0f;
    V3 il = world_to_local(wi, f.tangent, f.binormal, f.normal);
    V3 ol = world_to_local(wo, f.tangent, f.binormal, f.normal);
    if (il.z == 0.0f) return 0.0f;
    float p = 0.0f;
#pragma unroll 1
    for (int k = 0; k < m.n_lobes; ++k) p += lobe_pdf(m.lobe[k], il, ol);
    return p / static_cast<float>(m.n_lobes);
}

GR_D uint32_t count_lobes(const DevMaterial& m, uint32_t mask) {  // material.rs:245-253
    uint32_t c = 0;
    for (int k = 0; k < m.n_lobes; ++k)
        if (m.lobe[k].kind & mask) ++c;
    return c;
}

struct MaterialSample {
    V3 emission, radiance, outgoing;
    float pdf;
    uint32_t kind;
};

// material.rs:140-235.  u0 picks the lobe, u1 and u2 feed the lobe's sampler.
//
// The reference sums the chosen lobe's value and pdf first, then every other lobe's in
// index order.  One loop does all of it: step -1 is the chosen lobe, steps 0..n-1 the
// others, so Lobe::f and Lobe::pdf each have a single call site.  Inlined at every place
// the mixture uses them, they made the shading kernels too large for the instruction
// cache.  The first term is assigned rather than added to zero, so the sums (and the
// signs of zeros) are the reference's.
GR_D MaterialSample sample_world(const DevMaterial& m, V3 wi, const Frame& f, bool c2l, float u0, float u1,
                                 float u2) {
    V3 il = world_to_local(wi, f.tangent, f.binormal, f.normal);
    V3 emission = light_world(m, wi, f);
    int n = m.n_lobes;
    if (n == 0) return MaterialSample{emission, v3zero(), v3zero(), 1.0f, LOBE_NONE};
    int r = static_cast<int>(range_index(u0, static_cast<uint32_t>(n)));
    uint32_t kind = m.lobe[r].kind;
    V3 o;
    float given_pdf;
    int how = lobe_direction(m.lobe[r], il, u1, u2, o, given_pdf);
    V3 ow = local_to_world(o, f.tangent, f.binormal, f.normal);
    const bool mix = !(kind & LOBE_SPECULAR);
    bool gate = false;
    if (mix) {
        bool refl = (dot(wi, f.geom_normal) * dot(ow, f.geom_normal)) > 0.0f;
        // material.rs:203-206: the gate tests the chosen lobe's kind for every lobe (kept).
        gate = (refl && (kind & LOBE_REFLECTION)) || (!refl && (kind & LOBE_TRANSMISSION));
    }
    V3 radiance = v3zero();
    float pdf = 0.0f;
#pragma unroll 1
    for (int j = -1; j < n; ++j) {
        const bool first = j < 0;
        if (first ? how == SAMPLE_NONE : (!mix || j == r)) continue;
        const DevLobe& L = m.lobe[first ? r : j];
        float pk = first && how == SAMPLE_PDF_GIVEN ? given_pdf : lobe_pdf(L, il, o);
        pdf = first ? pk : pdf + pk;
        if (first || gate) {
            V3 fk = lobe_f(L, il, o, c2l);
            radiance = first ? fk : radiance + fk;
        }
    }
    pdf /= static_cast<float>(n);
    if (pdf == 0.0f) return MaterialSample{emission, v3zero(), ow, 1.0f, LOBE_NONE};
    return MaterialSample{emission, radiance, ow, pdf, kind};
}

}  // namespace gr
