// ORACLE — test infrastructure only (see ocore.hpp).  Parity unpinned.
//
// CPU restatement of the reference's src/material/: util.rs (Fresnel and microfacet
// distributions), lobes.rs (Disney diffuse/sheen, GGX specular, GTR1 clearcoat, GGX
// transmission, PerfectDiffuse, PerfectMirror), material.rs (the lobe mixture and the
// Disney builder) and lights.rs.  Random draws are explicit uniforms (u1, u2) in the
// order the reference draws them.
#pragma once

#include <memory>
#include <vector>

#include "ocore.hpp"

namespace orc {

// lobes.rs:25-40
enum LobeKind : uint32_t {
    LOBE_NONE = 0,
    LOBE_DIFFUSE = 1,
    LOBE_SPECULAR = 2,
    LOBE_GLOSSY = 4,
    LOBE_REFLECTION = 8,
    LOBE_TRANSMISSION = 16,
};

// ------------------------------------------------------------ material/util.rs
inline float fresnel_schlick_weight(float cos_theta) {  // util.rs:8-11
    float x = clamp_unit(1.0f - cos_theta);
    return x * x * x * x * x;
}
inline Vec fresnel_schlick(float cos_theta, const Vec& r0) {  // util.rs:13-15
    return r0.lerp(Vec::one(), fresnel_schlick_weight(cos_theta));
}
inline float fresnel_dielectric(float cos_theta_in, float ior) {  // util.rs:21-49
    bool entering = cos_theta_in > 0.0f;
    float eta_i, eta_t, c;
    if (entering) {
        eta_i = 1.0f;
        eta_t = ior;
        c = clamp_unit(cos_theta_in);
    } else {
        eta_i = ior;
        eta_t = 1.0f;
        c = clamp_unit(-cos_theta_in);
    }
    float sin_theta_in = std::sqrt(std::fmax(0.0f, 1.0f - c * c));
    float sin_theta_trans = eta_i / eta_t * sin_theta_in;
    if (sin_theta_trans >= 1.0f) return 1.0f;
    float cos_theta_trans = std::sqrt(std::fmax(0.0f, 1.0f - sin_theta_trans * sin_theta_trans));
    float r_parl = ((eta_t * c) - (eta_i * cos_theta_trans)) / ((eta_t * c) + (eta_i * cos_theta_trans));
    float r_perp = ((eta_i * c) - (eta_t * cos_theta_trans)) / ((eta_i * c) + (eta_t * cos_theta_trans));
    return (r_parl * r_parl + r_perp * r_perp) / 2.0f;
}

struct Fresnel {
    virtual ~Fresnel() {}
    virtual Vec fresnel(float cos_theta) const = 0;
};
struct DisneyFresnel : Fresnel {  // util.rs:56-78
    Vec color, spec_color;
    float ior, metallic;
    DisneyFresnel(float ior_, const Vec& c, float specular_tint, float metallic_)
        : color(c), ior(ior_), metallic(metallic_) {
        spec_color = Vec::one().lerp(c.tint(), specular_tint);
    }
    Vec fresnel(float cos_theta) const override {
        Vec dielectric = spec_color * fresnel_dielectric(cos_theta, ior);
        Vec conductor = fresnel_schlick(cos_theta, color);
        return dielectric.lerp(conductor, metallic);
    }
};
struct DielectricFresnel : Fresnel {  // util.rs:80-94
    float ior;
    explicit DielectricFresnel(float i) : ior(i) {}
    Vec fresnel(float cos_theta) const override { return Vec::one() * fresnel_dielectric(cos_theta, ior); }
};
struct SchlickFresnel : Fresnel {  // util.rs:96-110
    Vec r0;
    explicit SchlickFresnel(const Vec& r) : r0(r) {}
    Vec fresnel(float cos_theta) const override { return fresnel_schlick(cos_theta, r0); }
};

struct MicrofacetDistribution {
    virtual ~MicrofacetDistribution() {}
    virtual float d(const Vec& half) const = 0;
    virtual float g(const Vec& i, const Vec& o) const = 0;
    virtual Vec sample_half(const Vec& i, float u1, float u2) const = 0;
    virtual float pdf(const Vec& i, const Vec& half) const = 0;
};

// util.rs:119-251 (PBRT 3e TrowbridgeReitzDistribution + the Disney shader).
struct GgxDistribution : MicrofacetDistribution {
    float ax, ay;
    GgxDistribution(float roughness, float anisotropic) {
        float aspect = std::sqrt(1.0f - anisotropic * 0.9f);
        ax = std::fmax(0.001f, roughness * roughness / aspect);
        ay = std::fmax(0.001f, roughness * roughness * aspect);
    }
    float lambda(const Vec& v) const {  // util.rs:135-146
        float abs_tan_theta = std::fabs(v.tan_theta());
        if (std::isfinite(abs_tan_theta)) {
            float alpha = std::sqrt(v.cos2_phi() * (ax * ax) + v.sin2_phi() * (ay * ay));
            float a2t2 = (alpha * abs_tan_theta) * (alpha * abs_tan_theta);
            return (-1.0f + std::sqrt(1.0f + a2t2)) * 0.5f;
        }
        return 0.0f;
    }
    float g1(const Vec& v) const { return 1.0f / (1.0f + lambda(v)); }
    // util.rs:152-194 — PBRT's sample11 with its rational fit for the y slope.
    static void sample11(float cos_theta, float u1, float u2, float& sx, float& sy) {
        if (cos_theta > 0.9999f) {
            float r = std::sqrt(u1 / (1.0f - u1));
            float phi = TWO_PI * u2;
            sx = r * std::cos(phi);
            sy = r * std::sin(phi);
            return;
        }
        float sin_theta = std::sqrt(std::fmax(0.0f, 1.0f - cos_theta * cos_theta));
        float tan_theta = sin_theta / cos_theta;
        float g1 = 2.0f / (1.0f + std::sqrt(1.0f + tan_theta * tan_theta));
        float a = 2.0f * u1 / g1 - 1.0f;
        float tmp = std::fmin(1.0f / (a * a - 1.0f), 1e10f);
        float b = tan_theta;
        float d = std::sqrt(std::fmax(b * b * tmp * tmp - (a * a - b * b) * tmp, 0.0f));
        float slope_x_1 = b * tmp - d;
        float slope_x_2 = b * tmp + d;
        float slope_x = (a < 0.0f || slope_x_2 > 1.0f / tan_theta) ? slope_x_1 : slope_x_2;
        float s, u;
        if (u2 > 0.5f) {
            s = 1.0f;
            u = 2.0f * (u2 - 0.5f);
        } else {
            s = -1.0f;
            u = 2.0f * (0.5f - u2);
        }
        float z = (u * (u * (u * 0.27385f - 0.73369f) + 0.46341f)) /
                  (u * (u * (u * 0.093073f + 0.309420f) - 1.000000f) + 0.597999f);
        float slope_y = s * z * std::sqrt(1.0f + slope_x * slope_x);
        sx = slope_x;
        sy = slope_y;
    }
    float d(const Vec& half) const override {  // util.rs:198-208
        float tan2_theta = half.tan2_theta();
        if (std::isfinite(tan2_theta)) {
            float cos4_theta = half.cos2_theta() * half.cos2_theta();
            float e = (half.cos2_phi() / (ax * ax) + half.sin2_phi() / (ay * ay)) * tan2_theta;
            return 1.0f / (PI * ax * ay * cos4_theta * (1.0f + e) * (1.0f + e));
        }
        return 0.0f;
    }
    float g(const Vec& i, const Vec& o) const override { return 1.0f / (1.0f + lambda(i) + lambda(o)); }
    Vec sample_half(const Vec& i, float u1, float u2) const override {  // util.rs:214-240
        bool flip = i.z < 0.0f;
        Vec i_f = flip ? -i : i;
        Vec i_s = Vec(ax * i_f.x, ay * i_f.y, i_f.z).normalized();
        float cos_theta = i_s.cos_theta();
        float sx, sy;
        sample11(cos_theta, u1, u2, sx, sy);
        float cos_phi = i_s.cos_phi();
        float sin_phi = i_s.sin_phi();
        float sxr = ax * (cos_phi * sx - sin_phi * sy);
        float syr = ay * (sin_phi * sx + cos_phi * sy);
        Vec half = Vec(-sxr, -syr, 1.0f).normalized();
        return flip ? -half : half;
    }
    float pdf(const Vec& i, const Vec& half) const override {  // util.rs:242-250
        float cos_theta = i.cos_theta();
        if (cos_theta == 0.0f) return 0.0f;
        return d(half) * g1(i) * std::fabs(i.dot(half)) / std::fabs(cos_theta);
    }
};

// util.rs:255-309 (Burley 2012, GTR1).
struct Gtr1Distribution : MicrofacetDistribution {
    float alpha;
    explicit Gtr1Distribution(float clearcoat_gloss) : alpha(orc::lerp(0.1f, 0.001f, clearcoat_gloss)) {}
    float lambda(const Vec& v) const {  // util.rs:266-274
        float alpha_g = 0.25f;
        float cos_theta = v.abs_cos_theta();
        float alpha2 = alpha_g * alpha_g;
        float cos_theta2 = cos_theta * cos_theta;
        return 1.0f / (cos_theta + std::sqrt(alpha2 + cos_theta2 - (alpha2 * cos_theta2)));
    }
    float d(const Vec& half) const override {
        float alpha2 = alpha * alpha;
        float cos_theta = half.abs_cos_theta();
        return (alpha2 - 1.0f) / (PI * std::log(alpha2) * (1.0f + (alpha2 - 1.0f) * cos_theta * cos_theta));
    }
    float g(const Vec& i, const Vec& o) const override { return 1.0f / (1.0f + lambda(i) + lambda(o)); }
    // util.rs:291-303: the first draw is the azimuth, the second the elevation.
    Vec sample_half(const Vec& i, float u1, float u2) const override {
        float alpha2 = alpha * alpha;
        float phi = 2.0f * PI * u1;
        float cos_theta = std::sqrt(clamp_unit(1.0f - std::pow(alpha2, 1.0f - u2) / (1.0f - alpha2)));
        Vec h = Vec::from_spherical(cos_theta, phi);
        return h.is_local_same_hemisphere(i) ? h : -h;
    }
    float pdf(const Vec&, const Vec& half) const override { return d(half); }
};

// ----------------------------------------------------------- material/lobes.rs
struct LobeSample {
    Vec result, outgoing;
    float pdf;
    static LobeSample zero() { return LobeSample{Vec::zero(), Vec::zero(), 0.0f}; }
};

struct Lobe {
    virtual ~Lobe() {}
    virtual Vec f(const Vec& i, const Vec& o, bool camera_to_light) const = 0;
    virtual float pdf(const Vec& i, const Vec& o) const {  // lobes.rs:45-52
        if (!i.is_local_same_hemisphere(o)) return 0.0f;
        return cosine_hemisphere_pdf(o);
    }
    virtual LobeSample sample_f(const Vec& i, bool c2l, float u1, float u2) const {  // lobes.rs:54-68
        Vec o = cosine_sample_hemisphere(i.z < 0.0f, u1, u2);
        Vec result = f(i, o, c2l);
        float p = pdf(i, o);
        return LobeSample{result, o, p};
    }
    virtual uint32_t kind() const { return LOBE_DIFFUSE | LOBE_REFLECTION; }
};

// lobes.rs:76-116
struct DisneyDiffuseRefl : Lobe {
    Vec color, sheen_color;
    float roughness;
    DisneyDiffuseRefl(const Vec& c, float rough, float sheen, float sheen_tint, float diffuse_weight) {
        color = c * diffuse_weight;
        sheen_color = (sheen * diffuse_weight) * Vec::one().lerp(c.tint(), sheen_tint);
        roughness = rough;
    }
    Vec f(const Vec& i, const Vec& o, bool) const override {
        float f_in = fresnel_schlick_weight(i.abs_cos_theta());
        float f_out = fresnel_schlick_weight(o.abs_cos_theta());
        Vec diffuse = color * (FRAC_1_PI * (1.0f - 0.5f * f_in) * (1.0f - 0.5f * f_out));
        Vec half_unnorm = i + o;
        if (half_unnorm.is_exactly_zero()) return diffuse;
        Vec half = half_unnorm.normalized();
        float cos_theta_d = o.dot(half);
        float r_r = 2.0f * roughness * cos_theta_d * cos_theta_d;
        Vec retro = color * (FRAC_1_PI * r_r * (f_out + f_in + f_out * f_in * (r_r - 1.0f)));
        Vec sheen = sheen_color * fresnel_schlick_weight(cos_theta_d);
        return diffuse + (retro + sheen);
    }
};

// lobes.rs:126-189 — StandardMicrofacetRefl<Dist, Fresnel>.
struct StandardMicrofacetRefl : Lobe {
    std::unique_ptr<MicrofacetDistribution> microfacet;
    std::unique_ptr<Fresnel> fresnel;
    Vec color;
    Vec f(const Vec& i, const Vec& o, bool) const override {
        float cos_theta_in = i.abs_cos_theta();
        float cos_theta_out = o.abs_cos_theta();
        Vec half_unnorm = i + o;
        if (half_unnorm.is_exactly_zero() || cos_theta_in == 0.0f || cos_theta_out == 0.0f) return Vec::zero();
        Vec half = half_unnorm.normalized();
        Vec fr = fresnel->fresnel(o.dot(half));
        float d = microfacet->d(half);
        float g = microfacet->g(i, o);
        return color.comp_mult(fr) * (d * g / (4.0f * cos_theta_out * cos_theta_in));
    }
    float pdf(const Vec& i, const Vec& o) const override {
        if (!i.is_local_same_hemisphere(o)) return 0.0f;
        Vec half = (i + o).normalized();
        return microfacet->pdf(i, half) / (4.0f * i.dot(half));
    }
    LobeSample sample_f(const Vec& i, bool c2l, float u1, float u2) const override {
        if (i.z == 0.0f) return LobeSample::zero();
        Vec half = microfacet->sample_half(i, u1, u2);
        Vec o = i.reflect(half);
        if (!i.is_local_same_hemisphere(o)) return LobeSample::zero();
        Vec result = f(i, o, c2l);
        float p = microfacet->pdf(i, half) / (4.0f * i.dot(half));
        return LobeSample{result, o, p};
    }
    uint32_t kind() const override { return LOBE_GLOSSY | LOBE_REFLECTION; }
};

// lobes.rs:212-226
inline std::unique_ptr<Lobe> disney_specular_refl(const Vec& color, float roughness, float anisotropic,
                                                  float ior, float specular_tint, float metallic) {
    float ior_adjusted = std::fmax(ior, 1.01f);
    auto l = std::make_unique<StandardMicrofacetRefl>();
    l->microfacet = std::make_unique<GgxDistribution>(roughness, anisotropic);
    l->fresnel = std::make_unique<DisneyFresnel>(ior_adjusted, color, specular_tint, metallic);
    l->color = Vec::one();
    return l;
}
// lobes.rs:232-242
inline std::unique_ptr<Lobe> disney_clearcoat_refl(float clearcoat, float clearcoat_gloss) {
    auto l = std::make_unique<StandardMicrofacetRefl>();
    l->microfacet = std::make_unique<Gtr1Distribution>(clearcoat_gloss);
    l->fresnel = std::make_unique<SchlickFresnel>(0.04f * Vec::one());
    l->color = (0.25f * clearcoat) * Vec::one();
    return l;
}

// lobes.rs:246-393
struct DisneySpecularTrans : Lobe {
    GgxDistribution microfacet;
    DielectricFresnel fresnel;
    float ior;
    Vec color;
    DisneySpecularTrans(const Vec& c, float roughness, float anisotropic, float ior_)
        : microfacet(roughness, anisotropic), fresnel(std::fmax(ior_, 1.01f)),
          ior(std::fmax(ior_, 1.01f)), color(c) {}
    Vec f(const Vec& i, const Vec& o, bool camera_to_light) const override {
        if (i.is_local_same_hemisphere(o)) return Vec::zero();
        float cos_theta_in = i.cos_theta();
        float cos_theta_out = o.cos_theta();
        if (cos_theta_in == 0.0f || cos_theta_out == 0.0f) return Vec::zero();
        float eta = cos_theta_in > 0.0f ? ior : 1.0f / ior;
        Vec half_unnorm = i + (o * eta);
        Vec half = half_unnorm.z > 0.0f ? half_unnorm.normalized() : -half_unnorm.normalized();
        Vec fr = fresnel.fresnel(o.dot(half));
        float d = microfacet.d(half);
        float g = microfacet.g(i, o);
        float sqrt_denom = i.dot(half) + eta * o.dot(half);
        float factor = camera_to_light ? 1.0f : eta;
        Vec fresnel_inverse = Vec::one() - fr;
        return color.comp_mult(fresnel_inverse) *
               std::fabs(d * g * factor * factor * std::fabs(o.dot(half)) * std::fabs(i.dot(half)) /
                         (cos_theta_out * cos_theta_in * sqrt_denom * sqrt_denom));
    }
    // lobes.rs:321-349 — keeps the unnormalised half vector when half_unnorm.z > 0.
    float pdf(const Vec& i, const Vec& o) const override {
        if (i.is_local_same_hemisphere(o)) return 0.0f;
        float eta = i.cos_theta() > 0.0f ? ior : 1.0f / ior;
        Vec half_unnorm = i + (o * eta);
        Vec half = half_unnorm.z > 0.0f ? half_unnorm : -half_unnorm.normalized();
        float sqrt_denom = i.dot(half) + eta * o.dot(half);
        float dwh_dwi = std::fabs((eta * eta * o.dot(half)) / (sqrt_denom * sqrt_denom));
        return microfacet.pdf(i, half) * dwh_dwi;
    }
    LobeSample sample_f(const Vec& i, bool c2l, float u1, float u2) const override {
        if (i.z == 0.0f) return LobeSample::zero();
        Vec half = microfacet.sample_half(i, u1, u2);
        float eta = i.cos_theta() > 0.0f ? 1.0f / ior : ior;
        Vec o = i.refract(half, eta);
        if (o.is_exactly_zero()) return LobeSample::zero();
        Vec result = f(i, o, c2l);
        float p = pdf(i, o);
        return LobeSample{result, o, p};
    }
    uint32_t kind() const override { return LOBE_GLOSSY | LOBE_TRANSMISSION; }
};

// lobes.rs:401-414
struct PerfectDiffuse : Lobe {
    Vec f(const Vec&, const Vec&, bool) const override { return Vec(0.5f, 0.5f, 0.5f) * FRAC_1_PI; }
};
// lobes.rs:422-457
struct PerfectMirror : Lobe {
    Vec f(const Vec&, const Vec& o, bool) const override { return Vec::one() / o.abs_cos_theta(); }
    float pdf(const Vec&, const Vec&) const override { return 1.0f; }
    LobeSample sample_f(const Vec& i, bool c2l, float, float) const override {
        Vec o(-i.x, -i.y, i.z);
        return LobeSample{f(i, o, c2l), o, pdf(i, o)};
    }
    uint32_t kind() const override { return LOBE_SPECULAR | LOBE_REFLECTION; }
};

// -------------------------------------------------------- material/material.rs
// SurfaceProperties (geom/prim.rs:57-79).
struct SurfaceProperties {
    Vec normal, tangent, binormal, geom_normal;
    static SurfaceProperties zero() { return SurfaceProperties{}; }
};

struct MaterialSample {  // material.rs:12-18
    Vec emission, radiance, outgoing;
    float pdf;
    uint32_t kind;
};

struct DisneyParams {  // material.rs:256-290 (builder defaults)
    Vec base_color = Vec::one();
    float roughness = 0.5f, anisotropic = 0.0f, ior = 1.5f, metallic = 0.0f;
    float specular_trans = 0.0f, specular_tint = 0.0f, sheen = 0.0f, sheen_tint = 0.5f;
    float clearcoat = 0.0f, clearcoat_gloss = 0.1f;
};

struct Material {
    Vec display;
    bool has_light_ = false;
    Vec light_color;  // DiffuseAreaLight (lights.rs:11-22)
    std::vector<std::unique_ptr<Lobe>> lobes;

    static Material diffuse_light(const Vec& incandescence) {  // material.rs:27-33
        Material m;
        m.display = incandescence;
        m.has_light_ = true;
        m.light_color = incandescence;
        return m;
    }
    static Material diffuse() {
        Material m;
        m.display = Vec::one();
        m.lobes.push_back(std::make_unique<PerfectDiffuse>());
        return m;
    }
    static Material mirror() {
        Material m;
        m.display = Vec::one();
        m.lobes.push_back(std::make_unique<PerfectMirror>());
        return m;
    }
    // DisneyMaterialBuilder::build (material.rs:292-333)
    static Material disney(const DisneyParams& p) {
        Material m;
        float diffuse_weight = (1.0f - p.metallic) * (1.0f - p.specular_trans);
        float trans_weight = (1.0f - p.metallic) * p.specular_trans;
        if (diffuse_weight > 0.0f)
            m.lobes.push_back(std::make_unique<DisneyDiffuseRefl>(p.base_color, p.roughness, p.sheen,
                                                                  p.sheen_tint, diffuse_weight));
        if (p.ior > 1.0f)
            m.lobes.push_back(disney_specular_refl(p.base_color, p.roughness, p.anisotropic, p.ior,
                                                   p.specular_tint, p.metallic));
        if (p.clearcoat > 0.0f) m.lobes.push_back(disney_clearcoat_refl(p.clearcoat, p.clearcoat_gloss));
        if (trans_weight > 0.0f) {
            Vec c = trans_weight * p.base_color.sqrt();
            m.lobes.push_back(std::make_unique<DisneySpecularTrans>(c, p.roughness, p.anisotropic, p.ior));
        }
        m.display = p.base_color;
        return m;
    }

    bool has_light() const { return has_light_; }

    Vec l_world(const Vec& i, const SurfaceProperties& sp) const {  // lights.rs:15-21
        if (i.dot(sp.geom_normal) > 0.0f) return light_color;
        return Vec::zero();
    }

    // material.rs:66-93
    Vec f_world(const Vec& in_w, const Vec& out_w, const SurfaceProperties& sp, bool c2l) const {
        Vec il = in_w.world_to_local(sp.tangent, sp.binormal, sp.normal);
        Vec ol = out_w.world_to_local(sp.tangent, sp.binormal, sp.normal);
        bool reflect = (in_w.dot(sp.geom_normal) * out_w.dot(sp.geom_normal)) > 0.0f;
        Vec radiance = Vec::zero();
        for (const auto& lobe : lobes) {
            uint32_t k = lobe->kind();
            if ((reflect && (k & LOBE_REFLECTION)) || (!reflect && (k & LOBE_TRANSMISSION)))
                radiance = radiance + lobe->f(il, ol, c2l);
        }
        return radiance;
    }

    // material.rs:95-119
    float pdf_world(const Vec& in_w, const Vec& out_w, const SurfaceProperties& sp) const {
        if (lobes.empty()) return 0.0f;
        Vec il = in_w.world_to_local(sp.tangent, sp.binormal, sp.normal);
        Vec ol = out_w.world_to_local(sp.tangent, sp.binormal, sp.normal);
        if (il.z == 0.0f) return 0.0f;
        float p = 0.0f;
        for (const auto& lobe : lobes) p += lobe->pdf(il, ol);
        return p / static_cast<float>(lobes.size());
    }

    // material.rs:123-134
    Vec light_world(const Vec& in_w, const SurfaceProperties& sp) const {
        if (has_light_) return l_world(in_w, sp);
        return Vec::zero();
    }

    // material.rs:140-235.  u[0] picks the lobe, u[1], u[2] go to the lobe's sampler.
    MaterialSample sample_world(const Vec& in_w, const SurfaceProperties& sp, bool c2l,
                                const float u[3]) const {
        Vec il = in_w.world_to_local(sp.tangent, sp.binormal, sp.normal);
        Vec emission = has_light_ ? l_world(in_w, sp) : Vec::zero();
        if (lobes.empty()) return MaterialSample{emission, Vec::zero(), Vec::zero(), 1.0f, LOBE_NONE};
        uint32_t n = static_cast<uint32_t>(lobes.size());
        uint32_t r = range_index(u[0], n);
        const Lobe& lobe = *lobes[r];
        LobeSample s = lobe.sample_f(il, c2l, u[1], u[2]);
        Vec out_w = s.outgoing.local_to_world(sp.tangent, sp.binormal, sp.normal);
        Vec radiance = s.result;
        float pdf = s.pdf;
        uint32_t kind = lobe.kind();
        if (!(kind & LOBE_SPECULAR)) {
            for (uint32_t idx = 0; idx < n; ++idx)
                if (idx != r) pdf += lobes[idx]->pdf(il, s.outgoing);
        }
        pdf /= static_cast<float>(n);
        if (!(kind & LOBE_SPECULAR)) {
            bool reflect = (in_w.dot(sp.geom_normal) * out_w.dot(sp.geom_normal)) > 0.0f;
            for (uint32_t idx = 0; idx < n; ++idx) {
                // material.rs:203-206: the gate tests the *chosen* lobe's kind (kept).
                if (idx != r && ((reflect && (kind & LOBE_REFLECTION)) ||
                                 (!reflect && (kind & LOBE_TRANSMISSION))))
                    radiance = radiance + lobes[idx]->f(il, s.outgoing, c2l);
            }
        }
        if (pdf == 0.0f) return MaterialSample{emission, Vec::zero(), out_w, 1.0f, LOBE_NONE};
        return MaterialSample{emission, radiance, out_w, pdf, kind};
    }

    // material.rs:245-253
    uint32_t count_lobes(uint32_t mask) const {
        uint32_t c = 0;
        for (const auto& lobe : lobes)
            if (lobe->kind() & mask) ++c;
        return c;
    }
};

}  // namespace orc
