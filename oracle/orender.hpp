// ORACLE — test infrastructure only (see ocore.hpp).  Parity unpinned.
//
// CPU restatement of the reference's src/render/: integrators.rs (DisplayColor, the
// BSDF-sampling path tracer and the BDPT with uniform strategy weights), film.rs (jittered
// sample points, Mitchell splat), stage.rs (one pass per call) and exr.rs.
//
// Parameters replace the reference's compile-time constants; the defaults reproduce it:
//   PT:   max_depth 0 (unlimited), roulette when depth > 10, aggressive when depth > 20
//         (integrators.rs:36-37).
//   BDPT: max walk / path length 16, roulette when walk length >= 4 (integrators.rs:102-103).
// Extension, off by default: a constant environment radiance for escaped rays
// (the reference returns black, integrators.rs:90-92 and 210-225).
#pragma once

#include <cstdio>
#include <cstring>
#include <vector>

#include "ogeom.hpp"

namespace orc {

struct RenderSettings {
    int integrator = 0;  // 0 PT, 1 BDPT, 2 display colour
    uint32_t max_depth = 0;
    uint32_t rr_depth = 10;
    uint32_t rr_aggressive_depth = 20;
    uint64_t seed = 0;
    Vec environment;
};

struct Scene {
    std::vector<Material> materials;
    Bvh bvh;
    Vec environment;

    const Material& material_of(uint32_t prim) const { return materials[bvh.prims[prim].material]; }
    SurfaceProperties hit_props(const Ray& r, const Hit& h) const {
        return bvh.prims[h.prim].surface_props(r, h.component, h.dist, h.u, h.v);
    }
};

// ---------------------------------------------------------- path tracer
// integrators.rs:42-100.  Per segment `depth` the draws are dims
// DIM_CAMERA_WALK + 4*depth + {0: lobe, 1, 2: lobe sampler, 3: roulette}.
inline Vec integrate_pt(const Scene& sc, const Ray& initial, uint64_t key, const RenderSettings& rs) {
    uint32_t depth = 0;
    Vec light = Vec::zero();
    Vec throughput = Vec::one();
    Ray ray = initial;
    bool env = !sc.environment.is_exactly_zero();
    while (!throughput.is_exactly_zero() && (rs.max_depth == 0 || depth < rs.max_depth)) {
        Hit h = sc.bvh.intersect(ray);
        if (h.hit) {
            Vec incoming = -ray.direction;
            SurfaceProperties sp = sc.hit_props(ray, h);
            uint32_t base = DIM_CAMERA_WALK + 4 * depth;
            float u[3] = {uniform(key, base), uniform(key, base + 1), uniform(key, base + 2)};
            MaterialSample s = sc.material_of(h.prim).sample_world(incoming, sp, true, u);
            light = light + throughput.comp_mult(s.emission);
            throughput = throughput.comp_mult(s.radiance * (std::fabs(sp.normal.dot(s.outgoing)) / s.pdf));
            ray = Ray(ray.at(h.dist), s.outgoing).nudge();
            if (depth > rs.rr_depth || throughput.is_nearly_zero()) {
                float rv = uniform(key, base + 3);
                float prob_live = depth > rs.rr_aggressive_depth
                                      ? clamped_lerp(0.10f, 0.75f, throughput.luminance())
                                      : clamped_lerp(0.25f, 1.00f, throughput.luminance());
                if (rv < prob_live) throughput = throughput / prob_live;
                else throughput = Vec::zero();
            }
        } else {
            if (env) light = light + throughput.comp_mult(sc.environment);
            throughput = Vec::zero();
        }
        depth += 1;
    }
    return light;
}

// ----------------------------------------------------------------- BDPT
struct BdptVertex {  // integrators.rs:107-130
    Vec incoming, point;
    SurfaceProperties sp;
    Vec throughput, emission;
    uint32_t lobe_kind;
    bool connectible;
    uint32_t prim;  // NO_INDEX = escaped (usize::MAX)
    float pdf_forward, pdf_reverse;
    Vec escape_throughput;  // throughput before an escape (environment extension only)
};

inline float correct_shading_normal(const Vec& in_w, const Vec& out_w, const SurfaceProperties& sp, bool c2l) {
    if (c2l) return 1.0f;  // integrators.rs:232-251
    float num = std::fabs(in_w.dot(sp.normal)) * std::fabs(out_w.dot(sp.geom_normal));
    float denom = std::fabs(in_w.dot(sp.geom_normal)) * std::fabs(out_w.dot(sp.normal));
    if (denom == 0.0f) return 0.0f;
    return num / denom;
}

inline float convert_density(const Vec& prev, const Vec& next, const SurfaceProperties& nsp) {
    float dist = (next - prev).magnitude();  // integrators.rs:253-266
    if (dist == 0.0f) return 0.0f;
    Vec p2n = (next - prev) / dist;
    return std::fabs(nsp.normal.dot(p2n)) / (dist * dist);
}

// integrators.rs:138-229
inline void random_walk(const Scene& sc, const Ray& initial, const Vec& initial_tp, bool c2l, uint64_t key,
                        uint32_t dim_base, uint32_t max_len, uint32_t rr_len, std::vector<BdptVertex>& st) {
    Vec throughput = initial_tp;
    Ray ray = initial;
    while (!throughput.is_exactly_zero() && st.size() < max_len) {
        Hit h = sc.bvh.intersect(ray);
        if (h.hit) {
            Vec prev_tp = throughput;
            Vec hit_point = ray.at(h.dist);
            Vec incoming = -ray.direction;
            const Material& mat = sc.material_of(h.prim);
            SurfaceProperties sp = sc.hit_props(ray, h);
            uint32_t base = dim_base + 4 * static_cast<uint32_t>(st.size());
            float u[3] = {uniform(key, base), uniform(key, base + 1), uniform(key, base + 2)};
            MaterialSample s = mat.sample_world(incoming, sp, c2l, u);
            float pdf_reverse = mat.pdf_world(s.outgoing, incoming, sp);
            bool connectible = mat.count_lobes(LOBE_DIFFUSE | LOBE_GLOSSY) != 0;
            throughput = throughput.comp_mult(s.radiance * (std::fabs(sp.normal.dot(s.outgoing)) / s.pdf));
            throughput = throughput * correct_shading_normal(incoming, s.outgoing, sp, c2l);
            ray = Ray(ray.at(h.dist), s.outgoing).nudge();
            if (!st.empty()) {
                BdptVertex& last = st.back();
                last.pdf_reverse = pdf_reverse * convert_density(last.point, hit_point, sp);
            }
            st.push_back(BdptVertex{incoming, hit_point, sp, prev_tp, s.emission, s.kind, connectible, h.prim,
                                    s.pdf, 1.0f, Vec::zero()});
            if (st.size() >= rr_len || throughput.is_nearly_zero()) {
                float rv = uniform(key, base + 3);
                float prob_live = clamped_lerp(0.25f, 0.75f, throughput.luminance());
                if (rv < prob_live) throughput = throughput / prob_live;
                else throughput = Vec::zero();
            }
        } else {
            Vec escape = throughput;
            throughput = Vec::zero();
            st.push_back(BdptVertex{-ray.direction, Vec::zero(), SurfaceProperties::zero(), throughput, Vec::zero(),
                                    LOBE_NONE, false, NO_INDEX, 1.0f, 1.0f, escape});
        }
    }
}

// integrators.rs:269-343
inline Vec bdpt_connect(const Scene& sc, size_t cl, size_t ll, const std::vector<BdptVertex>& cs,
                        const std::vector<BdptVertex>& ls) {
    const BdptVertex& cv = cs[cl - 1];
    if (ll == 0) {
        if (cv.prim == NO_INDEX) return Vec::zero();
        return cv.throughput.comp_mult(cv.emission);
    }
    const BdptVertex& lv = ls[ll - 1];
    if (cv.prim == NO_INDEX || lv.prim == NO_INDEX) return Vec::zero();
    if (!cv.connectible || !lv.connectible) return Vec::zero();
    Vec c2l = (lv.point - cv.point).normalized();
    Vec l2c = -c2l;
    const Material& cm = sc.material_of(cv.prim);
    const Material& lm = sc.material_of(lv.prim);
    Vec connect_radiance = cm.f_world(cv.incoming, c2l, cv.sp, true);
    Vec connect_emission = ll == 1 ? lm.light_world(l2c, lv.sp) : lm.f_world(lv.incoming, l2c, lv.sp, false);
    float g = std::fabs(cv.sp.normal.dot(c2l));
    float cd = convert_density(cv.point, lv.point, lv.sp);
    Vec contrib = cv.throughput.comp_mult(connect_radiance).comp_mult(connect_emission).comp_mult(lv.throughput) *
                  (g * cd);
    if (contrib.is_nearly_zero()) return contrib;
    if (sc.bvh.visibility(cv.point, lv.point)) return contrib;
    return Vec::zero();
}

// integrators.rs:357-418.  Scenes without lights keep only the camera-only strategies
// (the reference panics in Bvh::sample_light there).  An escaped camera path adds
// throughput * environment with weight 1 (the only strategy that can produce it).
inline Vec integrate_bdpt(const Scene& sc, const Ray& initial, uint64_t key, const RenderSettings& rs,
                          std::vector<BdptVertex>& cs, std::vector<BdptVertex>& ls) {
    uint32_t max_len = rs.max_depth ? rs.max_depth : 16;
    uint32_t rr_len = rs.rr_depth;
    Vec light = Vec::zero();
    cs.clear();
    ls.clear();
    random_walk(sc, initial, Vec::one(), true, key, DIM_CAMERA_WALK, max_len, rr_len, cs);
    if (cs.empty()) return light;
    if (!sc.environment.is_exactly_zero() && cs.back().prim == NO_INDEX)
        light = light + cs.back().escape_throughput.comp_mult(sc.environment);
    bool have_light_path = false;
    if (!sc.bvh.light_indices.empty()) {
        float u[6];
        for (int k = 0; k < 6; ++k) u[k] = uniform(key, DIM_LIGHT_SAMPLE + k);
        LightSample lsmp = sc.bvh.sample_light(u);
        if (lsmp.point_pdf == 0.0f || lsmp.dir_pdf == 0.0f) return light;
        const Vec& light_dir = lsmp.ray.direction;
        const Material& lmat = sc.material_of(lsmp.prim);
        Vec initial_emission = lmat.light_world(light_dir, lsmp.sp) *
                               (std::fabs(lsmp.sp.geom_normal.dot(light_dir)) / (lsmp.point_pdf * lsmp.dir_pdf));
        ls.push_back(BdptVertex{Vec::zero(), lsmp.ray.origin, lsmp.sp, Vec::one() / lsmp.point_pdf, Vec::zero(),
                                LOBE_NONE, true, lsmp.prim, lsmp.point_pdf * lsmp.dir_pdf, 1.0f, Vec::zero()});
        random_walk(sc, lsmp.ray.nudge(), initial_emission, false, key, DIM_LIGHT_WALK, max_len, rr_len, ls);
        have_light_path = true;
    }
    size_t lmax = have_light_path ? ls.size() : 0;
    for (size_t c = 1; c <= cs.size(); ++c) {
        for (size_t l = 0; l <= lmax; ++l) {
            if (c + l > max_len) continue;
            Vec L = bdpt_connect(sc, c, l, cs, ls);
            float w = 1.0f / static_cast<float>(c + l);  // integrators.rs:345-354
            light = light + (L * w);
        }
    }
    return light;
}

// integrators.rs:18-34
inline Vec integrate_display(const Scene& sc, const Ray& ray) {
    Hit h = sc.bvh.intersect(ray);
    if (h.hit) return sc.material_of(h.prim).display;
    return Vec::zero();
}

// ----------------------------------------------------------------- film
struct FilmSample {
    Vec color;
    float s, t;
};
struct FilmPixel {
    Vec accum;
    float weight;
};
constexpr float FILTER_WIDTH = 2.0f;  // film.rs:8

// film.rs:55-76: jitter U(-2, 2) around each pixel centre, row draw first.
inline void sample_point(uint32_t width, uint32_t height, uint32_t row, uint32_t col, uint64_t key, float& s,
                         float& t) {
    float widthf = static_cast<float>(width), heightf = static_cast<float>(height);
    float row_cont = 0.5f + static_cast<float>(row);
    float col_cont = 0.5f + static_cast<float>(col);
    float row_j = row_cont + (-FILTER_WIDTH + (FILTER_WIDTH - -FILTER_WIDTH) * uniform(key, DIM_JITTER_ROW));
    float col_j = col_cont + (-FILTER_WIDTH + (FILTER_WIDTH - -FILTER_WIDTH) * uniform(key, DIM_JITTER_COL));
    s = lerp(-1.0f, 1.0f, col_j / widthf);
    t = lerp(-1.0f, 1.0f, row_j / heightf);
}

// film.rs:78-114 — serial Mitchell splat in sample order.
inline void report_samples(uint32_t width, uint32_t height, const std::vector<FilmSample>& samples,
                           std::vector<FilmPixel>& pixels) {
    float widthf = static_cast<float>(width), heightf = static_cast<float>(height);
    long long last_col = static_cast<long long>(width) - 1, last_row = static_cast<long long>(height) - 1;
    for (const FilmSample& s : samples) {
        float col_cont = lerp(0.0f, widthf, 0.5f * (s.s + 1.0f));
        float row_cont = lerp(0.0f, heightf, 0.5f * (s.t + 1.0f));
        float col_discr = col_cont - 0.5f;
        float row_discr = row_cont - 0.5f;
        long long min_col = clamp<long long>(static_cast<long long>(std::ceil(col_discr - FILTER_WIDTH)), 0, last_col);
        long long max_col = clamp<long long>(static_cast<long long>(std::floor(col_discr + FILTER_WIDTH)), 0, last_col);
        long long min_row = clamp<long long>(static_cast<long long>(std::ceil(row_discr - FILTER_WIDTH)), 0, last_row);
        long long max_row = clamp<long long>(static_cast<long long>(std::floor(row_discr + FILTER_WIDTH)), 0, last_row);
        for (long long y = min_row; y <= max_row; ++y) {
            for (long long x = min_col; x <= max_col; ++x) {
                FilmPixel& p = pixels[static_cast<size_t>(y) * width + static_cast<size_t>(x)];
                float w = mitchell_filter2(static_cast<float>(x) - col_discr, static_cast<float>(y) - row_discr,
                                           FILTER_WIDTH);
                p.accum = p.accum + (s.color * w);
                p.weight += w;
            }
        }
    }
}

// exr.rs:37-199 — header, line-offset table, then B, G, R float planes per
// scanline, the bottom row first.
inline std::vector<unsigned char> exr_bytes(uint32_t width, uint32_t height, const std::vector<FilmPixel>& px) {
    std::vector<unsigned char> b;
    auto i32 = [&](int32_t v) {
        uint32_t u = static_cast<uint32_t>(v);
        for (int k = 0; k < 4; ++k) b.push_back(static_cast<unsigned char>((u >> (8 * k)) & 0xFF));
    };
    auto u64 = [&](uint64_t v) {
        for (int k = 0; k < 8; ++k) b.push_back(static_cast<unsigned char>((v >> (8 * k)) & 0xFF));
    };
    auto f32 = [&](float f) {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        i32(static_cast<int32_t>(u));
    };
    auto str = [&](const char* s) {
        while (*s) b.push_back(static_cast<unsigned char>(*s++));
        b.push_back(0);
    };
    i32(20000630);
    i32(2);
    str("channels");
    str("chlist");
    i32(2 * 3 + 16 * 3 + 1);
    for (const char* ch : {"B", "G", "R"}) {
        str(ch);
        i32(2);
        i32(0);
        i32(1);
        i32(1);
    }
    b.push_back(0);
    str("compression");
    str("compression");
    i32(1);
    b.push_back(0);
    int32_t window[4] = {0, 0, static_cast<int32_t>(width) - 1, static_cast<int32_t>(height) - 1};
    str("dataWindow");
    str("box2i");
    i32(16);
    for (int32_t v : window) i32(v);
    str("displayWindow");
    str("box2i");
    i32(16);
    for (int32_t v : window) i32(v);
    str("lineOrder");
    str("lineOrder");
    i32(1);
    b.push_back(0);
    str("pixelAspectRatio");
    str("float");
    i32(4);
    f32(1.0f);
    str("screenWindowCenter");
    str("v2f");
    i32(8);
    f32(0.0f);
    f32(0.0f);
    str("screenWindowWidth");
    str("float");
    i32(4);
    f32(static_cast<float>(width));
    b.push_back(0);
    size_t line_size = 4 + 4 + static_cast<size_t>(width) * 4 * 3;
    size_t data_offset = b.size() + 8 * static_cast<size_t>(height);
    for (uint32_t y = 0; y < height; ++y) u64(data_offset + y * line_size);
    for (uint32_t y = 0; y < height; ++y) {
        i32(static_cast<int32_t>(y));
        i32(static_cast<int32_t>(line_size - 8));
        size_t first = static_cast<size_t>(height - y - 1) * width;
        for (int ch = 2; ch >= 0; --ch)
            for (uint32_t i = 0; i < width; ++i) {
                const FilmPixel& p = px[first + i];
                f32(p.accum[ch] / p.weight);
            }
    }
    return b;
}

}  // namespace orc
