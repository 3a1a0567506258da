// ORACLE — test infrastructure only (see ocore.hpp).  Parity unpinned.
//
// The C ABI of include/gammaray.h over the CPU restatement, so one test harness can
// drive the CUDA library and this checker the same way.  Passes run the per-pixel
// integrator on all host threads (the reference's rayon par_iter_mut,
// render/stage.rs:30) and splat serially (render/film.rs:78-114).
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../include/gammaray.h"
#include "orender.hpp"

using namespace orc;

namespace {

thread_local std::string g_last_error;

gr_status fail(gr_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

unsigned thread_count() {
    const char* env = std::getenv("GR_ORACLE_THREADS");
    if (env && std::atoi(env) > 0) return static_cast<unsigned>(std::atoi(env));
    unsigned n = std::thread::hardware_concurrency();
    return n ? n : 1;
}

template <class F>
void parallel_for(size_t n, F&& fn) {
    unsigned nt = thread_count();
    if (nt <= 1 || n < 256) {
        for (size_t i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<size_t> next(0);
    std::atomic<bool> failed(false);
    std::exception_ptr err;
    std::mutex err_mu;
    auto worker = [&]() {
        const size_t chunk = 64;
        for (;;) {
            size_t b = next.fetch_add(chunk);
            if (b >= n || failed.load()) return;
            size_t e = b + chunk < n ? b + chunk : n;
            try {
                for (size_t i = b; i < e; ++i) fn(i);
            } catch (...) {
                std::lock_guard<std::mutex> g(err_mu);
                err = std::current_exception();
                failed = true;
                return;
            }
        }
    };
    std::vector<std::thread> ts;
    for (unsigned t = 0; t < nt; ++t) ts.emplace_back(worker);
    for (auto& t : ts) t.join();
    if (err) std::rethrow_exception(err);
}

Vec v3(const float* p) { return Vec(p[0], p[1], p[2]); }
void put3(float* p, const Vec& v) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}

bool make_material(const gr_material_desc& d, Material& out, std::string& err) {
    switch (d.kind) {
        case GR_MATERIAL_DISNEY: {
            DisneyParams p;
            p.base_color = v3(d.base_color);
            p.roughness = d.roughness;
            p.anisotropic = d.anisotropic;
            p.ior = d.ior;
            p.metallic = d.metallic;
            p.specular_trans = d.specular_trans;
            p.specular_tint = d.specular_tint;
            p.sheen = d.sheen;
            p.sheen_tint = d.sheen_tint;
            p.clearcoat = d.clearcoat;
            p.clearcoat_gloss = d.clearcoat_gloss;
            out = Material::disney(p);
            return true;
        }
        case GR_MATERIAL_DIFFUSE_LIGHT:
            out = Material::diffuse_light(v3(d.incandescence));
            return true;
        case GR_MATERIAL_DIFFUSE:
            out = Material::diffuse();
            return true;
        case GR_MATERIAL_MIRROR:
            out = Material::mirror();
            return true;
        default:
            err = "unknown material kind " + std::to_string(d.kind);
            return false;
    }
}

SurfaceProperties frame_of(const gr_frame& f) {
    return SurfaceProperties{v3(f.normal), v3(f.tangent), v3(f.binormal), v3(f.geom_normal)};
}

}  // namespace

struct gr_scene {
    Scene sc;
    double build_seconds = 0.0;
};

struct gr_film {
    uint32_t width = 0, height = 0;
    std::vector<FilmPixel> pixels;
    std::vector<Vec> splat;  // light-tracing splat sums (BDPT extension); empty until used
    uint32_t passes = 0;
    bool has_splat() const { return !splat.empty(); }
    float splat_scale() const { return passes ? 1.0f / static_cast<float>(passes) : 0.0f; }
};

extern "C" {

const char* gr_last_error(void) { return g_last_error.c_str(); }
int gr_abi_version(void) { return GR_ABI_VERSION; }
const char* gr_backend_name(void) { return "oracle-cpu"; }

void gr_material_disney_defaults(gr_material_desc* o) {
    std::memset(o, 0, sizeof(*o));
    DisneyParams p;
    o->kind = GR_MATERIAL_DISNEY;
    put3(o->base_color, p.base_color);
    o->roughness = p.roughness;
    o->anisotropic = p.anisotropic;
    o->ior = p.ior;
    o->metallic = p.metallic;
    o->specular_trans = p.specular_trans;
    o->specular_tint = p.specular_tint;
    o->sheen = p.sheen;
    o->sheen_tint = p.sheen_tint;
    o->clearcoat = p.clearcoat;
    o->clearcoat_gloss = p.clearcoat_gloss;
}

void gr_render_params_default(int32_t integrator, gr_render_params* o) {
    std::memset(o, 0, sizeof(*o));
    o->integrator = integrator;
    o->spp = 1;
    if (integrator == GR_INTEGRATOR_BDPT) {
        o->max_depth = 16;
        o->rr_depth = 4;
        o->rr_aggressive_depth = 0;
    } else {
        o->max_depth = 0;
        o->rr_depth = 10;
        o->rr_aggressive_depth = 20;
    }
}

gr_status gr_scene_create(const gr_scene_desc* desc, gr_scene** out) {
    if (!desc || !out) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    auto t0 = std::chrono::steady_clock::now();
    auto s = std::make_unique<gr_scene>();
    std::vector<bool> has_light;
    for (uint32_t i = 0; i < desc->num_materials; ++i) {
        Material m;
        std::string err;
        if (!make_material(desc->materials[i], m, err)) return fail(GR_ERR_INVALID_ARGUMENT, err);
        has_light.push_back(m.has_light());
        s->sc.materials.push_back(std::move(m));
    }
    std::vector<Prim> prims;
    for (uint32_t i = 0; i < desc->num_prims; ++i) {
        const gr_prim_desc& d = desc->prims[i];
        if (d.material >= desc->num_materials)
            return fail(GR_ERR_INVALID_ARGUMENT, "prim " + std::to_string(i) + ": material index out of range");
        Prim p;
        p.material = static_cast<int>(d.material);
        if (d.kind == GR_PRIM_SPHERE) {
            if (!(d.radius > 0.0f)) return fail(GR_ERR_INVALID_ARGUMENT, "sphere radius must be > 0");
            p.is_sphere = true;
            p.radius = d.radius;
            p.origin = v3(d.center);
        } else if (d.kind == GR_PRIM_MESH) {
            if (d.num_tris == 0 || !d.vertices || !d.tri_vertices)
                return fail(GR_ERR_INVALID_ARGUMENT, "mesh " + std::to_string(i) + " has no triangles");
            for (uint32_t v = 0; v < d.num_vertices; ++v) p.vertices.push_back(v3(d.vertices + 3 * v));
            for (uint32_t v = 0; v < d.num_normals; ++v) p.normals.push_back(v3(d.normals + 3 * v));
            for (uint32_t v = 0; v < d.num_uvs; ++v) p.uvs.push_back(Vec(d.uvs[2 * v], d.uvs[2 * v + 1], 0.0f));
            uint32_t zero_uv = static_cast<uint32_t>(p.uvs.size());
            if (!d.tri_uvs) p.uvs.push_back(Vec::zero());
            for (uint32_t t = 0; t < d.num_tris; ++t) {
                Tri tr;
                tr.a = d.tri_vertices[3 * t];
                tr.b = d.tri_vertices[3 * t + 1];
                tr.c = d.tri_vertices[3 * t + 2];
                if (tr.a >= d.num_vertices || tr.b >= d.num_vertices || tr.c >= d.num_vertices)
                    return fail(GR_ERR_INVALID_ARGUMENT, "vertex index out of range");
                if (d.tri_normals && d.tri_normals[3 * t] != GR_NO_INDEX) {
                    tr.an = d.tri_normals[3 * t];
                    tr.bn = d.tri_normals[3 * t + 1];
                    tr.cn = d.tri_normals[3 * t + 2];
                    if (tr.an >= d.num_normals || tr.bn >= d.num_normals || tr.cn >= d.num_normals)
                        return fail(GR_ERR_INVALID_ARGUMENT, "normal index out of range");
                } else {
                    tr.an = tr.bn = tr.cn = NO_INDEX;
                }
                if (d.tri_uvs) {
                    tr.at = d.tri_uvs[3 * t];
                    tr.bt = d.tri_uvs[3 * t + 1];
                    tr.ct = d.tri_uvs[3 * t + 2];
                    if (tr.at >= d.num_uvs || tr.bt >= d.num_uvs || tr.ct >= d.num_uvs)
                        return fail(GR_ERR_INVALID_ARGUMENT, "uv index out of range");
                } else {
                    tr.at = tr.bt = tr.ct = zero_uv;
                }
                p.tris.push_back(tr);
            }
            p.finish_mesh();
        } else {
            return fail(GR_ERR_INVALID_ARGUMENT, "unknown prim kind");
        }
        prims.push_back(std::move(p));
    }
    s->sc.environment = v3(desc->environment);
    s->sc.bvh.build(std::move(prims), has_light);
    s->build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = s.release();
    return GR_OK;
}

// FNV-1a over the flattened tree (depth-first, left child first, as bvh.rs:310-337
// lays it out): each node's box, then a leaf's count and (prim, component) ids, or an
// inner node's tag.  The GPU library hashes its build the same way.
static uint64_t tree_hash(const Bvh& b) {
    uint64_t h = 1469598103934665603ull;
    auto add = [&](const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) {
            h ^= c[i];
            h *= 1099511628211ull;
        }
    };
    for (const LinearNode& nd : b.nodes) {
        const float box[6] = {nd.bbox.min.x, nd.bbox.min.y, nd.bbox.min.z, nd.bbox.max.x, nd.bbox.max.y, nd.bbox.max.z};
        add(box, sizeof(box));
        if (nd.num_components > 0) {
            const uint32_t tag = 1, count = static_cast<uint32_t>(nd.num_components);
            add(&tag, 4);
            add(&count, 4);
            for (size_t j = 0; j < nd.num_components; ++j) {
                const uint32_t pc[2] = {b.components[nd.offset + j].first, b.components[nd.offset + j].second};
                add(pc, sizeof(pc));
            }
        } else {
            const uint32_t tag = 0;
            add(&tag, 4);
        }
    }
    return h;
}

gr_status gr_scene_plan(const gr_scene_desc* desc, gr_scene_info* o) {
    gr_scene* s = nullptr;
    gr_status st = gr_scene_create(desc, &s);
    if (st != GR_OK) return st;
    st = gr_scene_get_info(s, o);
    if (st == GR_OK) o->tree_hash = tree_hash(s->sc.bvh);
    delete s;
    return st;
}

gr_status gr_scene_destroy(gr_scene* s) {
    delete s;
    return GR_OK;
}

gr_status gr_scene_get_info(const gr_scene* s, gr_scene_info* o) {
    if (!s || !o) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(o, 0, sizeof(*o));
    o->num_components = s->sc.bvh.components.size();
    o->num_binary_nodes = s->sc.bvh.nodes.size();
    o->num_lights = static_cast<uint32_t>(s->sc.bvh.light_indices.size());
    o->bvh_width = 2;
    o->build_seconds = s->build_seconds;
    return GR_OK;
}

gr_status gr_scene_last_stats(const gr_scene* s, gr_render_stats* o) {
    if (!s || !o) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(o, 0, sizeof(*o));
    return GR_OK;
}

gr_status gr_film_create(uint32_t w, uint32_t h, gr_film** out) {
    if (!out || w == 0 || h == 0) return fail(GR_ERR_INVALID_ARGUMENT, "film size must be > 0");
    auto f = new gr_film;
    f->width = w;
    f->height = h;
    f->pixels.assign(static_cast<size_t>(w) * h, FilmPixel{Vec::zero(), 0.0f});
    *out = f;
    return GR_OK;
}
gr_status gr_film_destroy(gr_film* f) {
    delete f;
    return GR_OK;
}
gr_status gr_film_clear(gr_film* f) {
    if (!f) return fail(GR_ERR_INVALID_ARGUMENT, "null film");
    std::fill(f->pixels.begin(), f->pixels.end(), FilmPixel{Vec::zero(), 0.0f});
    f->splat.clear();
    f->passes = 0;
    return GR_OK;
}
gr_status gr_film_read(const gr_film* f, float* accum, float* weight) {
    if (!f) return fail(GR_ERR_INVALID_ARGUMENT, "null film");
    for (size_t i = 0; i < f->pixels.size(); ++i) {
        if (accum) put3(accum + 3 * i, f->pixels[i].accum);
        if (weight) weight[i] = f->pixels[i].weight;
    }
    return GR_OK;
}
gr_status gr_film_read_splat(const gr_film* f, float* splat) {
    if (!f || !splat) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    for (size_t i = 0; i < f->pixels.size(); ++i) put3(splat + 3 * i, f->has_splat() ? f->splat[i] : Vec::zero());
    return GR_OK;
}
gr_status gr_film_resolve(const gr_film* f, float* rgb) {
    if (!f || !rgb) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    for (size_t i = 0; i < f->pixels.size(); ++i) {
        Vec v = f->pixels[i].accum / f->pixels[i].weight;
        if (f->has_splat()) v = v + f->splat[i] * f->splat_scale();
        put3(rgb + 3 * i, v);
    }
    return GR_OK;
}
gr_status gr_film_write_exr(const gr_film* f, const char* path) {
    if (!f || !path) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<unsigned char> b =
        exr_bytes(f->width, f->height, f->pixels, f->has_splat() ? &f->splat : nullptr, f->splat_scale());
    std::ofstream os(path, std::ios::binary);
    if (!os) return fail(GR_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    os.write(reinterpret_cast<const char*>(b.data()), static_cast<std::streamsize>(b.size()));
    return os ? GR_OK : fail(GR_ERR_INTERNAL, "write failed");
}
gr_status gr_film_passes(const gr_film* f, uint32_t* p) {
    if (!f || !p) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    *p = f->passes;
    return GR_OK;
}

static gr_status check_params(const gr_render_params* p) {
    if (!p) return fail(GR_ERR_INVALID_ARGUMENT, "null params");
    if (p->integrator < 0 || p->integrator > 2) return fail(GR_ERR_INVALID_ARGUMENT, "unknown integrator");
    if (p->integrator != GR_INTEGRATOR_BDPT && (p->mis != 0 || p->light_tracing != 0))
        return fail(GR_ERR_INVALID_ARGUMENT, "mis and light_tracing apply to the BDPT integrator only");
    if (p->integrator == GR_INTEGRATOR_BDPT && p->max_depth > 16)
        return fail(GR_ERR_INVALID_ARGUMENT, "BDPT max_depth must be <= 16");
    return GR_OK;
}

static Camera make_camera(const gr_camera* c) {
    return Camera(c->focal_length, c->horizontal_aperture, c->vertical_aperture, c->f_stop, c->rotate[0],
                  Vec(c->rotate[1], c->rotate[2], c->rotate[3]), v3(c->translate));
}

// One Stage::trace pass (render/stage.rs:23-36) without the splat.  With the
// light-tracing extension, `splats` receives each sample's light-tracing splats, in
// sample order.
static void trace_pass(const gr_scene* s, const Camera& cam, const gr_render_params* p, uint32_t w, uint32_t h,
                       uint32_t pass, std::vector<FilmSample>& samples, std::vector<Splat>* splats = nullptr) {
    RenderSettings rs;
    rs.integrator = p->integrator;
    rs.max_depth = p->max_depth;
    rs.rr_depth = p->rr_depth;
    rs.rr_aggressive_depth = p->rr_aggressive_depth;
    rs.seed = p->seed;
    rs.mis = p->mis != 0;
    rs.light_tracing = p->light_tracing != 0;
    const PinholeView view = PinholeView::of(cam);
    samples.assign(static_cast<size_t>(w) * h, FilmSample{Vec::zero(), 0.0f, 0.0f});
    std::vector<std::vector<Splat>> per_sample(rs.light_tracing && splats ? samples.size() : 0);
    parallel_for(samples.size(), [&](size_t i) {
        thread_local std::vector<BdptVertex> cs, ls;
        uint32_t row = static_cast<uint32_t>(i / w), col = static_cast<uint32_t>(i % w);
        uint64_t key = path_key(p->seed, pass, static_cast<uint32_t>(i));
        FilmSample& fs = samples[i];
        sample_point(w, h, row, col, key, fs.s, fs.t);
        Ray ray = cam.compute_ray(fs.s, fs.t);
        if (p->integrator == GR_INTEGRATOR_PATH_TRACER) fs.color = integrate_pt(s->sc, ray, key, rs);
        else if (p->integrator == GR_INTEGRATOR_BDPT)
            fs.color = integrate_bdpt(s->sc, ray, key, rs, cs, ls, &view, w, h,
                                      per_sample.empty() ? nullptr : &per_sample[i]);
        else fs.color = integrate_display(s->sc, ray);
    });
    if (splats) {
        splats->clear();
        for (auto& v : per_sample) splats->insert(splats->end(), v.begin(), v.end());
    }
}

gr_status gr_render(gr_scene* s, const gr_camera* c, const gr_render_params* p, gr_film* f) {
    if (!s || !c || !f) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    gr_status st = check_params(p);
    if (st != GR_OK) return st;
    Camera cam = make_camera(c);
    std::vector<FilmSample> samples;
    std::vector<Splat> splats;
    const bool lt = p->integrator == GR_INTEGRATOR_BDPT && p->light_tracing != 0;
    try {
        for (uint32_t k = 0; k < p->spp; ++k) {
            trace_pass(s, cam, p, f->width, f->height, p->first_pass + k, samples, lt ? &splats : nullptr);
            report_samples(f->width, f->height, samples, f->pixels);
            if (lt) {
                if (f->splat.empty()) f->splat.assign(f->pixels.size(), Vec::zero());
                for (const Splat& sp : splats) f->splat[sp.pixel] = f->splat[sp.pixel] + sp.value;
            }
            f->passes += 1;
        }
    } catch (const StackOverflow& e) {
        return fail(GR_ERR_STACK_OVERFLOW, e.what());
    }
    return GR_OK;
}

gr_status gr_render_samples(gr_scene* s, const gr_camera* c, const gr_render_params* p, uint32_t w, uint32_t h,
                            float* out) {
    if (!s || !c || !out || w == 0 || h == 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
    gr_status st = check_params(p);
    if (st != GR_OK) return st;
    std::vector<FilmSample> samples;
    try {
        trace_pass(s, make_camera(c), p, w, h, p->first_pass, samples);
    } catch (const StackOverflow& e) {
        return fail(GR_ERR_STACK_OVERFLOW, e.what());
    }
    for (size_t i = 0; i < samples.size(); ++i) {
        out[5 * i] = samples[i].s;
        out[5 * i + 1] = samples[i].t;
        put3(out + 5 * i + 2, samples[i].color);
    }
    return GR_OK;
}

static void put_hit(gr_hit& o, const Hit& h) {
    if (h.hit) {
        o.t = h.dist;
        o.prim = static_cast<int32_t>(h.prim);
        o.component = static_cast<int32_t>(h.component);
        o.u = h.u;
        o.v = h.v;
    } else {
        o.t = 0.0f;
        o.prim = -1;
        o.component = -1;
        o.u = o.v = 0.0f;
    }
}

gr_status gr_trace_rays(gr_scene* s, const float* rays, uint64_t n, gr_hit* hits) {
    if (!s || (n && (!rays || !hits))) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    try {
        parallel_for(n, [&](size_t i) {
            Ray r(v3(rays + 6 * i), v3(rays + 6 * i + 3));
            put_hit(hits[i], s->sc.bvh.intersect(r));
        });
    } catch (const StackOverflow& e) {
        return fail(GR_ERR_STACK_OVERFLOW, e.what());
    }
    return GR_OK;
}

gr_status gr_trace_rays_dev(gr_scene*, const float*, uint64_t, gr_hit*, void*) {
    return fail(GR_ERR_UNSUPPORTED, "the CPU restatement has no device buffers");
}

gr_status gr_intersect_naive(gr_scene* s, const float* rays, uint64_t n, gr_hit* hits) {
    if (!s || (n && (!rays || !hits))) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    parallel_for(n, [&](size_t i) {
        Ray r(v3(rays + 6 * i), v3(rays + 6 * i + 3));
        put_hit(hits[i], s->sc.bvh.intersect_naive(r));
    });
    return GR_OK;
}

gr_status gr_visibility(gr_scene* s, const float* pairs, uint64_t n, uint8_t* visible) {
    if (!s || (n && (!pairs || !visible))) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    try {
        parallel_for(n, [&](size_t i) {
            visible[i] = s->sc.bvh.visibility(v3(pairs + 6 * i), v3(pairs + 6 * i + 3)) ? 1 : 0;
        });
    } catch (const StackOverflow& e) {
        return fail(GR_ERR_STACK_OVERFLOW, e.what());
    }
    return GR_OK;
}

gr_status gr_sample_light(gr_scene* s, const float* u, uint64_t n, gr_light_sample* out) {
    if (!s || (n && (!u || !out))) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    if (s->sc.bvh.light_indices.empty()) return fail(GR_ERR_INVALID_ARGUMENT, "scene has no lights");
    for (uint64_t i = 0; i < n; ++i) {
        LightSample ls = s->sc.bvh.sample_light(u + 6 * i);
        gr_light_sample& o = out[i];
        put3(o.origin, ls.ray.origin);
        put3(o.direction, ls.ray.direction);
        put3(o.normal, ls.sp.normal);
        put3(o.tangent, ls.sp.tangent);
        put3(o.binormal, ls.sp.binormal);
        put3(o.geom_normal, ls.sp.geom_normal);
        o.prim = static_cast<int32_t>(ls.prim);
        o.point_pdf = ls.point_pdf;
        o.dir_pdf = ls.dir_pdf;
    }
    return GR_OK;
}

gr_status gr_bsdf_eval(const gr_material_desc* md, uint64_t n, const gr_frame* fr, const float* in,
                       const float* out, int32_t c2l, float* f) {
    Material m;
    std::string err;
    if (!md || !make_material(*md, m, err)) return fail(GR_ERR_INVALID_ARGUMENT, err.empty() ? "null" : err);
    for (uint64_t i = 0; i < n; ++i)
        put3(f + 3 * i, m.f_world(v3(in + 3 * i), v3(out + 3 * i), frame_of(fr[i]), c2l != 0));
    return GR_OK;
}

gr_status gr_bsdf_pdf(const gr_material_desc* md, uint64_t n, const gr_frame* fr, const float* in,
                      const float* out, float* pdf) {
    Material m;
    std::string err;
    if (!md || !make_material(*md, m, err)) return fail(GR_ERR_INVALID_ARGUMENT, err.empty() ? "null" : err);
    for (uint64_t i = 0; i < n; ++i) pdf[i] = m.pdf_world(v3(in + 3 * i), v3(out + 3 * i), frame_of(fr[i]));
    return GR_OK;
}

gr_status gr_bsdf_sample_batch(const gr_material_desc* md, uint64_t n, const gr_frame* fr, const float* in,
                               const float* u, int32_t c2l, gr_bsdf_sample* o) {
    Material m;
    std::string err;
    if (!md || !make_material(*md, m, err)) return fail(GR_ERR_INVALID_ARGUMENT, err.empty() ? "null" : err);
    for (uint64_t i = 0; i < n; ++i) {
        MaterialSample s = m.sample_world(v3(in + 3 * i), frame_of(fr[i]), c2l != 0, u + 3 * i);
        put3(o[i].emission, s.emission);
        put3(o[i].radiance, s.radiance);
        put3(o[i].outgoing, s.outgoing);
        o[i].pdf = s.pdf;
        o[i].kind = s.kind;
    }
    return GR_OK;
}

gr_status gr_light_eval(const gr_material_desc* md, uint64_t n, const gr_frame* fr, const float* in, float* L) {
    Material m;
    std::string err;
    if (!md || !make_material(*md, m, err)) return fail(GR_ERR_INVALID_ARGUMENT, err.empty() ? "null" : err);
    for (uint64_t i = 0; i < n; ++i) put3(L + 3 * i, m.light_world(v3(in + 3 * i), frame_of(fr[i])));
    return GR_OK;
}

gr_status gr_render_batch(const gr_job* jobs, uint32_t n, const gr_batch_options*) {
    if (n && !jobs) return fail(GR_ERR_INVALID_ARGUMENT, "null jobs");
    for (uint32_t i = 0; i < n; ++i) {
        gr_status st = gr_render(jobs[i].scene, &jobs[i].camera, &jobs[i].params, jobs[i].film);
        if (st != GR_OK) return st;
    }
    return GR_OK;
}

gr_status gr_batch_autotune(const gr_job*, uint32_t, gr_batch_options* out) {
    if (!out) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(out, 0, sizeof(*out));
    return GR_OK;
}

gr_status gr_batch_release(void) { return GR_OK; }  // the CPU restatement caches nothing

gr_status gr_batch_last_stats(gr_render_stats* out) {
    if (!out) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(out, 0, sizeof(*out));
    return GR_OK;
}

gr_status gr_server_create(const gr_server_options*, gr_server**) {
    return fail(GR_ERR_UNSUPPORTED, "serving is a device feature");
}
gr_status gr_server_destroy(gr_server*) { return fail(GR_ERR_UNSUPPORTED, "serving is a device feature"); }
gr_status gr_server_submit(gr_server*, const gr_request*, uint64_t*) {
    return fail(GR_ERR_UNSUPPORTED, "serving is a device feature");
}
gr_status gr_server_step(gr_server*, double) { return fail(GR_ERR_UNSUPPORTED, "serving is a device feature"); }
gr_status gr_server_poll(gr_server*, uint64_t, gr_request_status*) {
    return fail(GR_ERR_UNSUPPORTED, "serving is a device feature");
}
gr_status gr_server_cancel(gr_server*, uint64_t) { return fail(GR_ERR_UNSUPPORTED, "serving is a device feature"); }
gr_status gr_server_snapshot(gr_server*, uint64_t, float*, float*, uint32_t*) {
    return fail(GR_ERR_UNSUPPORTED, "serving is a device feature");
}
gr_status gr_server_get_info(gr_server*, gr_server_info*) {
    return fail(GR_ERR_UNSUPPORTED, "serving is a device feature");
}
gr_status gr_server_take(gr_server*, uint64_t, float*, float*) {
    return fail(GR_ERR_UNSUPPORTED, "serving is a device feature");
}

}  // extern "C"
