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
    bool mis = false;            // BDPT extension: power-heuristic strategy weights
    bool light_tracing = false;  // BDPT extension: light-walk vertices splatted via the camera
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
    // MIS extension: PBRT-convention area pdfs of generating this vertex from its
    // predecessor on its own walk (afwd) and from its successor (arev), and whether the
    // lobe sampled here was specular (delta).
    float afwd = 0.0f, arev = 0.0f;
    bool delta = false;
};

// Solid-angle pdf `pdf` at `from` of the direction toward `to`, as an area density at
// `to` (surface with geometric normal ng).
inline float to_area(float pdf, const Vec& from, const Vec& to, const Vec& ng) {
    Vec v = to - from;
    float d2 = v.dot(v);
    if (d2 == 0.0f) return 0.0f;
    return pdf * (std::fabs(ng.dot(v)) / std::sqrt(d2)) / d2;
}

// The pinhole camera seen from the scene, for the light-tracing strategy and the
// camera's sampling pdf: its position, the world directions of its x, y, z axes (the
// camera matrix is a rotation and a translation, camera.rs:42-61) and the [-1, 1]^2
// image-plane window at distance 1 (camera.rs:76-97).
struct PinholeView {
    Vec pos, axis[3];
    float wx = 1.0f, wy = 1.0f, area = 4.0f;

    static PinholeView of(const Camera& c) {
        PinholeView v;
        v.pos = c.xform.transform(Vec::zero());
        for (int i = 0; i < 3; ++i) v.axis[i] = Vec(c.xform.m[i][0], c.xform.m[i][1], c.xform.m[i][2]);
        c.window_max(v.wx, v.wy);
        v.area = 4.0f * v.wx * v.wy;
        return v;
    }
    // Film position (s, t) of world point p, its distance and the cosine between the
    // viewing axis and the direction to p.  False when p is behind the camera or outside
    // the window.
    bool project(const Vec& p, float& s, float& t, float& dist, float& cos_view) const {
        Vec v = p - pos;
        float cx = v.dot(axis[0]), cy = v.dot(axis[1]), cz = v.dot(axis[2]);
        if (!(cz < 0.0f)) return false;
        s = (cx / -cz) / wx;
        t = (cy / -cz) / wy;
        dist = v.magnitude();
        cos_view = -cz / dist;
        return s >= -1.0f && s <= 1.0f && t >= -1.0f && t <= 1.0f;
    }
    // Solid-angle pdf of a camera ray at angle acos(cos_view) off the axis when rays are
    // spread uniformly over the window: 1 / (area cos^3).
    float dir_pdf(float cos_view) const { return 1.0f / (area * cos_view * cos_view * cos_view); }
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
// start / start_pdf (MIS extension only): the point the walk leaves from (camera or
// light point) and the solid-angle pdf of the initial direction.
inline void random_walk(const Scene& sc, const Ray& initial, const Vec& initial_tp, bool c2l, uint64_t key,
                        uint32_t dim_base, uint32_t max_len, uint32_t rr_len, std::vector<BdptVertex>& st,
                        const Vec& start = Vec::zero(), float start_pdf = 0.0f) {
    Vec throughput = initial_tp;
    Ray ray = initial;
    Vec prev_point = start;
    float dir_pdf = start_pdf;
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
            const bool delta = (s.kind & LOBE_SPECULAR) != 0;
            if (!st.empty()) {
                BdptVertex& last = st.back();
                last.pdf_reverse = pdf_reverse * convert_density(last.point, hit_point, sp);
                last.arev = to_area(delta ? 0.0f : pdf_reverse, hit_point, last.point, last.sp.geom_normal);
            }
            st.push_back(BdptVertex{incoming, hit_point, sp, prev_tp, s.emission, s.kind, connectible, h.prim,
                                    s.pdf, 1.0f, Vec::zero()});
            st.back().afwd = to_area(dir_pdf, prev_point, hit_point, sp.geom_normal);
            st.back().delta = delta;
            prev_point = hit_point;
            dir_pdf = delta ? 0.0f : s.pdf;
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

// ------------------------------------------- BDPT extension: MIS and light tracing
// Off by default; reference mode keeps integrators.rs:345-354's uniform 1 / (c + l).
// Multiple importance sampling with the power heuristic over all strategies of a path
// (Veach 1997, eq. 10.9 with beta = 2), in the ratio form of PBRT 3e section 16.3.4:
// per vertex the area pdfs of generating it along its own walk (afwd) and from the other
// side (arev), ratios of neighbouring strategies' pdfs chained outwards from the
// connection, delta (specular) vertices skipped and zero pdfs counted as 1.  The
// strategies are c camera-walk vertices and l light-walk vertices, c + l <= max_len,
// plus, with light tracing, c = 0: light-walk vertex y connected straight to the pinhole
// camera and splatted at its film position.

// Area pdf with which Bvh::sample_light picks point p of light prim `prim`
// (bvh.rs:481-496, mesh.rs:310-327, sphere.rs:103-111).
inline float light_point_pdf(const Scene& sc, uint32_t prim) {
    const Prim& P = sc.bvh.prims[prim];
    float pdf = P.is_sphere ? 1.0f / (4.0f * PI * P.radius * P.radius) : 1.0f / P.area;
    return pdf / static_cast<float>(sc.bvh.light_indices.size());
}

// Pdf of a light emitting toward w (cosine about the geometric normal, prim.rs:37-51).
inline float light_dir_pdf(const SurfaceProperties& sp, const Vec& w) {
    float c = sp.geom_normal.dot(w);
    return c > 0.0f ? c * FRAC_1_PI : 0.0f;
}

// Weight of strategy (c, l) given the reverse pdfs the connection implies for the last
// vertex of each walk and the one before it (z_rev, zm_rev; y_rev, ym_rev).
// lt_possible: the light-tracing strategy can produce this path (its first camera
// vertex projects inside the window and light tracing is on).
inline float mis_weight(const std::vector<BdptVertex>& cs, const std::vector<BdptVertex>& ls, size_t c, size_t l,
                        float z_rev, float zm_rev, float y_rev, float ym_rev, bool lt_possible) {
    auto remap = [](float x) { return x != 0.0f ? x : 1.0f; };
    float sum = 0.0f, r = 1.0f;
    for (size_t k = c; k-- > 0;) {  // move camera vertices to the light walk, last first
        float rev = k + 1 == c ? z_rev : (k + 2 == c ? zm_rev : cs[k].arev);
        r *= remap(rev) / remap(cs[k].afwd);
        bool here = k + 1 == c ? false : cs[k].delta;
        bool before = k == 0 ? false : cs[k - 1].delta;
        if (k == 0 && !lt_possible) continue;  // the strategy with no camera-walk vertex
        if (!here && !before) sum += r * r;
    }
    r = 1.0f;
    for (size_t k = l; k-- > 0;) {  // move light vertices to the camera walk, last first
        float rev = k + 1 == l ? y_rev : (k + 2 == l ? ym_rev : ls[k].arev);
        r *= remap(rev) / remap(ls[k].afwd);
        bool here = k + 1 == l ? false : ls[k].delta;
        bool before = k == 0 ? false : ls[k - 1].delta;
        if (!here && !before) sum += r * r;
    }
    return 1.0f / (1.0f + sum);
}

// MIS weight of camera strategy (c >= 1, l >= 0) for a non-zero connection.
inline float strategy_weight(const Scene& sc, const PinholeView& view, const std::vector<BdptVertex>& cs,
                             const std::vector<BdptVertex>& ls, size_t c, size_t l, bool lt_possible) {
    const BdptVertex& z = cs[c - 1];
    const Material& zm = sc.material_of(z.prim);
    float z_rev = 0.0f, zm_rev = 0.0f, y_rev = 0.0f, ym_rev = 0.0f;
    if (l == 0) {  // the camera walk hit a light
        z_rev = light_point_pdf(sc, z.prim);
        if (c >= 2) zm_rev = to_area(light_dir_pdf(z.sp, z.incoming), z.point, cs[c - 2].point, cs[c - 2].sp.geom_normal);
    } else {
        const BdptVertex& y = ls[l - 1];
        const Material& ym = sc.material_of(y.prim);
        Vec w_yz = (z.point - y.point).normalized();
        float pz = l == 1 ? light_dir_pdf(y.sp, w_yz) : ym.pdf_world(y.incoming, w_yz, y.sp);
        z_rev = to_area(pz, y.point, z.point, z.sp.geom_normal);
        if (c >= 2) zm_rev = to_area(zm.pdf_world(-w_yz, z.incoming, z.sp), z.point, cs[c - 2].point,
                                     cs[c - 2].sp.geom_normal);
        y_rev = to_area(zm.pdf_world(z.incoming, -w_yz, z.sp), z.point, y.point, y.sp.geom_normal);
        if (l >= 2) ym_rev = to_area(ym.pdf_world(w_yz, y.incoming, y.sp), y.point, ls[l - 2].point,
                                     ls[l - 2].sp.geom_normal);
    }
    (void)view;
    return mis_weight(cs, ls, c, l, z_rev, zm_rev, y_rev, ym_rev, lt_possible);
}

struct Splat {
    uint32_t pixel;
    Vec value;
};

// integrators.rs:357-418.  Scenes without lights keep only the camera-only strategies
// (the reference panics in Bvh::sample_light there).  An escaped camera path adds
// throughput * environment with weight 1 (the only strategy that can produce it).
// With rs.light_tracing, light-tracing contributions are appended to `splats` (film
// pixel, value) for a film of width x height.
inline Vec integrate_bdpt(const Scene& sc, const Ray& initial, uint64_t key, const RenderSettings& rs,
                          std::vector<BdptVertex>& cs, std::vector<BdptVertex>& ls, const PinholeView* view = nullptr,
                          uint32_t width = 0, uint32_t height = 0, std::vector<Splat>* splats = nullptr) {
    uint32_t max_len = rs.max_depth ? rs.max_depth : 16;
    uint32_t rr_len = rs.rr_depth;
    const bool ext = rs.mis || rs.light_tracing;
    Vec light = Vec::zero();
    cs.clear();
    ls.clear();
    float cam_pdf = 0.0f;
    if (ext) cam_pdf = view->dir_pdf(initial.direction.dot(-view->axis[2]));
    random_walk(sc, initial, Vec::one(), true, key, DIM_CAMERA_WALK, max_len, rr_len, cs, initial.origin, cam_pdf);
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
        ls.back().afwd = lsmp.point_pdf;
        random_walk(sc, lsmp.ray.nudge(), initial_emission, false, key, DIM_LIGHT_WALK, max_len, rr_len, ls,
                    lsmp.ray.origin, lsmp.dir_pdf);
        have_light_path = true;
    }
    size_t lmax = have_light_path ? ls.size() : 0;
    // Can the light-tracing strategy produce paths through this camera walk's first hit?
    bool lt_possible = false;
    if (rs.light_tracing && cs[0].prim != NO_INDEX) {
        float s, t, d, cv;
        lt_possible = view->project(cs[0].point, s, t, d, cv);
    }
    for (size_t c = 1; c <= cs.size(); ++c) {
        for (size_t l = 0; l <= lmax; ++l) {
            if (c + l > max_len) continue;
            Vec L = bdpt_connect(sc, c, l, cs, ls);
            float w;
            if (!rs.mis) w = 1.0f / static_cast<float>(c + l + (rs.light_tracing ? 1 : 0));
            else w = L.is_exactly_zero() ? 0.0f : strategy_weight(sc, *view, cs, ls, c, l, lt_possible);
            light = light + (L * w);
        }
    }
    if (rs.light_tracing && splats) {  // c = 0: light-walk vertex -> camera
        for (size_t l = 1; l <= lmax && l <= max_len; ++l) {
            const BdptVertex& y = ls[l - 1];
            if (y.prim == NO_INDEX || !y.connectible) continue;
            float s, t, dist, cv;
            if (!view->project(y.point, s, t, dist, cv)) continue;
            Vec w_yc = (view->pos - y.point) / dist;
            const Material& ym = sc.material_of(y.prim);
            Vec F = l == 1 ? ym.light_world(w_yc, y.sp) : ym.f_world(y.incoming, w_yc, y.sp, false);
            // We / pdf for a pinhole: 1 / (area cos^3 dist^2) (PBRT 3e section 16.1.1)
            float g = std::fabs(y.sp.normal.dot(w_yc)) / (view->area * cv * cv * cv * dist * dist);
            Vec L = y.throughput.comp_mult(F) * g;
            if (L.is_nearly_zero()) continue;
            if (!sc.bvh.visibility(view->pos, y.point)) continue;
            float w;
            if (!rs.mis) {
                w = 1.0f / static_cast<float>(l + 1);
            } else {
                float y_rev = to_area(view->dir_pdf(cv), view->pos, y.point, y.sp.geom_normal);
                float ym_rev = l >= 2 ? to_area(ym.pdf_world(w_yc, y.incoming, y.sp), y.point, ls[l - 2].point,
                                                ls[l - 2].sp.geom_normal)
                                      : 0.0f;
                w = mis_weight(cs, ls, 0, l, 0.0f, 0.0f, y_rev, ym_rev, true);
            }
            uint32_t col = std::min(width - 1, static_cast<uint32_t>(std::floor(0.5f * (s + 1.0f) * width)));
            uint32_t row = std::min(height - 1, static_cast<uint32_t>(std::floor(0.5f * (t + 1.0f) * height)));
            splats->push_back(Splat{row * width + col, L * w});
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
// `splat` (light-tracing extension): per-pixel splat sums added as splat * splat_scale.
inline std::vector<unsigned char> exr_bytes(uint32_t width, uint32_t height, const std::vector<FilmPixel>& px,
                                            const std::vector<Vec>* splat = nullptr, float splat_scale = 0.0f) {
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
                float v = p.accum[ch] / p.weight;
                if (splat) v = v + (*splat)[first + i][ch] * splat_scale;
                f32(v);
            }
    }
    return b;
}

}  // namespace orc
