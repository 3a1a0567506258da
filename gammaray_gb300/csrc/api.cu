// C ABI of libgammaray_gpu.so (include/gammaray.h): handle management, uploads and
// the host side of every entry point.  All device work of a scene runs on the
// scene's own stream; host-buffer calls copy in, launch and copy out on that stream.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <fstream>
#include <memory>

#include "runtime.hpp"

namespace gr {

static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }

static gr_status fail(gr_status s, const std::string& msg) {
    g_err = msg;
    return s;
}

DeviceWork& device_work() {
    static DeviceWork work[64];
    int dev = 0;
    cudaGetDevice(&dev);
    return work[dev < 0 || dev >= 64 ? 0 : dev];
}

gr_status sync_check(cudaStream_t st, const char* what, uint32_t bounce, uint32_t n) {
    static const double limit = [] {
        const char* e = std::getenv("GR_SYNC_CHECK");
        return e ? std::atof(e) : 0.0;
    }();
    if (limit <= 0.0) return GR_OK;
    cudaEvent_t ev;
    GR_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    GR_CUDA_TRY(cudaEventRecord(ev, st));
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t q = cudaEventQuery(ev);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) {
            cudaEventDestroy(ev);
            return fail(GR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(q));
        }
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > limit) {
            std::string msg = std::string(what) + " did not finish within " + std::to_string(limit) + " s (bounce " +
                              std::to_string(bounce) + ", capacity " + std::to_string(n) + ")";
            std::fprintf(stderr, "gammaray: %s\n", msg.c_str());
            cudaEventDestroy(ev);  // released once the work before it completes
            return fail(GR_ERR_TIMEOUT, msg);
        }
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    cudaEventDestroy(ev);
    return GR_OK;
}

template <class T>
static gr_status upload(DevBuf& b, const T& v, cudaStream_t st, uint64_t& total) {
    if (v.empty()) return GR_OK;
    size_t bytes = v.size() * sizeof(v[0]);
    GR_CUDA_TRY(b.ensure(bytes));
    GR_CUDA_TRY(cudaMemcpyAsync(b.ptr, v.data(), bytes, cudaMemcpyHostToDevice, st));
    total += bytes;
    return GR_OK;
}

// Camera::new (core/camera.rs:42-61): xform = translation * rotation (row vectors).
DevCamera make_camera(const gr_camera& c) {
    float T[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {c.translate[0], c.translate[1], c.translate[2], 1}};
    float r = c.rotate[0], ix = c.rotate[1], iy = c.rotate[2], iz = c.rotate[3];
    float R[4][4];  // core/matrix.rs:97-121
    R[0][0] = 1.0f - 2.0f * (iy * iy + iz * iz);
    R[0][1] = 2.0f * (ix * iy + iz * r);
    R[0][2] = 2.0f * (iz * ix - iy * r);
    R[0][3] = 0.0f;
    R[1][0] = 2.0f * (ix * iy - iz * r);
    R[1][1] = 1.0f - 2.0f * (iz * iz + ix * ix);
    R[1][2] = 2.0f * (iy * iz + ix * r);
    R[1][3] = 0.0f;
    R[2][0] = 2.0f * (iz * ix + iy * r);
    R[2][1] = 2.0f * (iy * iz - ix * r);
    R[2][2] = 1.0f - 2.0f * (iy * iy + ix * ix);
    R[2][3] = 0.0f;
    R[3][0] = R[3][1] = R[3][2] = 0.0f;
    R[3][3] = 1.0f;
    DevCamera d;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float s = T[i][0] * R[0][j];
            s = s + T[i][1] * R[1][j];
            s = s + T[i][2] * R[2][j];
            s = s + T[i][3] * R[3][j];
            d.m[i][j] = s;
        }
    d.wx = c.horizontal_aperture / (c.focal_length * 2.0f);  // camera.rs:76-79
    d.wy = c.vertical_aperture / (c.focal_length * 2.0f);
    return d;
}

gr_status check_render_params(const gr_render_params* p) {
    if (!p) return fail(GR_ERR_INVALID_ARGUMENT, "null params");
    if (p->integrator < 0 || p->integrator > 2) return fail(GR_ERR_INVALID_ARGUMENT, "unknown integrator");
    if (p->integrator == GR_INTEGRATOR_BDPT && p->max_depth > 16)
        return fail(GR_ERR_INVALID_ARGUMENT, "BDPT max_depth must be <= 16");
    if (p->integrator != GR_INTEGRATOR_BDPT && (p->mis || p->light_tracing))
        return fail(GR_ERR_INVALID_ARGUMENT, "mis / light_tracing apply to BDPT only");
    return GR_OK;
}

// Scratch copy-in / copy-out helper for the host-buffer query calls.
struct Scratch {
    std::vector<DevBuf*> bufs;
    ~Scratch() {
        for (DevBuf* b : bufs) delete b;
    }
    void* get(size_t bytes, cudaError_t& e) {
        DevBuf* b = new DevBuf();
        bufs.push_back(b);
        e = b->ensure(bytes ? bytes : 16);
        return b->ptr;
    }
};

}  // namespace gr

using namespace gr;

#define GR_TRY(expr)                      \
    do {                                  \
        gr_status s__ = (expr);           \
        if (s__ != GR_OK) return s__;     \
    } while (0)

namespace {
std::mutex g_scene_holders_mu;  // gr_scene::holders and destroy_pending

void scene_free(gr_scene* s) {
    { std::lock_guard<std::mutex> busy(s->mu); }  // a render on another thread ends first
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    cudaStream_t st = s->stream;
    delete s;
    if (st) cudaStreamDestroy(st);
}
}  // namespace

namespace gr {
void scene_retain(gr_scene* s) {
    std::lock_guard<std::mutex> g(g_scene_holders_mu);
    ++s->holders;
}

void scene_release(gr_scene* s) {
    bool last;
    {
        std::lock_guard<std::mutex> g(g_scene_holders_mu);
        last = --s->holders == 0 && s->destroy_pending;
    }
    if (last) scene_free(s);
}
}  // namespace gr

extern "C" {

const char* gr_last_error(void) { return g_err.c_str(); }
int gr_abi_version(void) { return GR_ABI_VERSION; }
const char* gr_backend_name(void) { return "cuda-sm_103a"; }

void gr_material_disney_defaults(gr_material_desc* o) {
    std::memset(o, 0, sizeof(*o));
    o->kind = GR_MATERIAL_DISNEY;  // material.rs:276-290
    o->base_color[0] = o->base_color[1] = o->base_color[2] = 1.0f;
    o->roughness = 0.5f;
    o->ior = 1.5f;
    o->sheen_tint = 0.5f;
    o->clearcoat_gloss = 0.1f;
}

void gr_render_params_default(int32_t integrator, gr_render_params* o) {
    std::memset(o, 0, sizeof(*o));
    o->integrator = integrator;
    o->spp = 1;
    if (integrator == GR_INTEGRATOR_BDPT) {  // integrators.rs:102-103
        o->max_depth = 16;
        o->rr_depth = 4;
    } else {  // integrators.rs:36-37
        o->rr_depth = 10;
        o->rr_aggressive_depth = 20;
    }
}

gr_status gr_scene_create(const gr_scene_desc* desc, gr_scene** out) {
    if (!desc || !out) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    auto t0 = std::chrono::steady_clock::now();
    std::unique_ptr<gr_scene> s(new gr_scene());
    std::string err;
    if (!build_scene(*desc, s->host, err)) return fail(GR_ERR_INVALID_ARGUMENT, err);
    GR_CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    GR_CUDA_TRY(cudaEventCreate(&s->ev0));
    GR_CUDA_TRY(cudaEventCreate(&s->ev1));
    HostBuild& h = s->host;
    SceneBuffers& b = s->buf;
    cudaStream_t st = s->stream;
    uint64_t total = 0;
    if (h.device_build) {
        uint32_t num_wide = 0, stack_depth = 0;
        GR_TRY(build_bvh_device(h, b, st, num_wide, stack_depth, total));
        h.num_wide_nodes = num_wide;
        h.stack_depth = stack_depth;
    } else {
        GR_TRY(upload(b.nodes, h.nodes, st, total));
        GR_TRY(upload(b.prims, h.prims, st, total));
        GR_TRY(upload(b.tri_nidx, h.tri_normal_idx, st, total));
        GR_TRY(upload(b.tri_uvidx, h.tri_uv_idx, st, total));
    }
    GR_TRY(upload(b.normals, h.normals, st, total));
    GR_TRY(upload(b.uvs, h.uvs, st, total));
    GR_TRY(upload(b.prim_material, h.prim_material, st, total));
    GR_TRY(upload(b.materials, h.materials, st, total));
    GR_TRY(upload(b.lights, h.lights, st, total));
    GR_TRY(upload(b.light_tris, h.light_tris, st, total));
    GR_TRY(upload(b.light_nidx, h.light_tri_normal_idx, st, total));
    GR_TRY(upload(b.light_uvidx, h.light_tri_uv_idx, st, total));
    GR_TRY(upload(b.light_cdf, h.light_cdf, st, total));
    GR_CUDA_TRY(cudaStreamSynchronize(st));
    DeviceScene& d = s->dev;
    d.nodes = b.nodes.as<float4>();
    d.prims = b.prims.as<float4>();
    d.tri_normal_idx = h.any_normals ? b.tri_nidx.as<uint32_t>() : nullptr;
    d.tri_uv_idx = h.any_uvs ? b.tri_uvidx.as<uint32_t>() : nullptr;
    d.normals = b.normals.as<float>();
    d.uvs = b.uvs.as<float>();
    d.prim_material = b.prim_material.as<uint32_t>();
    d.materials = b.materials.as<DevMaterial>();
    d.lights = b.lights.as<LightRec>();
    d.light_tris = b.light_tris.as<float4>();
    bool light_n = false, light_uv = false;
    for (uint32_t v : h.light_tri_normal_idx) light_n |= v != NO_INDEX;
    for (uint32_t v : h.light_tri_uv_idx) light_uv |= v != NO_INDEX;
    d.light_tri_normal_idx = light_n ? b.light_nidx.as<uint32_t>() : nullptr;
    d.light_tri_uv_idx = light_uv ? b.light_uvidx.as<uint32_t>() : nullptr;
    d.light_cdf = b.light_cdf.as<float>();
    d.num_lights = static_cast<uint32_t>(h.lights.size());
    d.num_components = static_cast<uint32_t>(h.num_components);
    d.width = h.width;
    d.stack_depth = h.stack_depth;
    d.step_budget = 8u * d.num_components + 4096u;
    if (const char* e = std::getenv("GR_STEP_BUDGET")) {
        long v = std::atol(e);
        if (v > 0) d.step_budget = static_cast<uint32_t>(std::min<long>(v, 0x7FFFFFFFL));
    }
    d.env[0] = desc->environment[0];
    d.env[1] = desc->environment[1];
    d.env[2] = desc->environment[2];
    d.has_env = (d.env[0] != 0.0f || d.env[1] != 0.0f || d.env[2] != 0.0f) ? 1 : 0;
    s->device_bytes = total;
    s->build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = s.release();
    return GR_OK;
}

static uint64_t planned_bytes(const HostBuild& h) {
    // A device build's node count is known only after it runs: at most one wide node
    // per component.
    const uint64_t nodes = h.device_build ? h.num_components * 8 * h.width * 4 : h.nodes.size() * 4;
    return nodes + h.prims.size() * 4 + (h.tri_normal_idx.size() + h.tri_uv_idx.size()) * 4 +
           (h.normals.size() + h.uvs.size()) * 4 + h.prim_material.size() * 4 + h.materials.size() * sizeof(DevMaterial) +
           h.lights.size() * sizeof(LightRec) + h.light_tris.size() * 4 +
           (h.light_tri_normal_idx.size() + h.light_tri_uv_idx.size()) * 4 + h.light_cdf.size() * 4;
}

gr_status gr_scene_plan(const gr_scene_desc* desc, gr_scene_info* o) {
    if (!desc || !o) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    auto t0 = std::chrono::steady_clock::now();
    HostBuild h;
    std::string err;
    if (!build_scene(*desc, h, err, true)) return fail(GR_ERR_INVALID_ARGUMENT, err);
    std::memset(o, 0, sizeof(*o));
    o->num_components = h.num_components;
    o->num_binary_nodes = h.num_binary_nodes;
    o->num_wide_nodes = h.num_wide_nodes;
    o->device_bytes = planned_bytes(h);
    o->num_lights = static_cast<uint32_t>(h.lights.size());
    o->bvh_width = h.width;
    o->build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    o->tree_hash = h.tree_hash;
    o->stack_depth = h.stack_depth;
    return GR_OK;
}

gr_status gr_scene_destroy(gr_scene* s) {
    if (!s) return GR_OK;
    {
        std::lock_guard<std::mutex> g(g_scene_holders_mu);
        if (s->holders) {  // freed by the server when its last request lets go
            s->destroy_pending = true;
            return GR_OK;
        }
    }
    scene_free(s);
    return GR_OK;
}

gr_status gr_scene_get_info(const gr_scene* s, gr_scene_info* o) {
    if (!s || !o) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(o, 0, sizeof(*o));
    o->num_components = s->host.num_components;
    o->num_binary_nodes = s->host.num_binary_nodes;
    o->num_wide_nodes = s->host.num_wide_nodes;
    o->device_bytes = s->device_bytes;
    o->num_lights = static_cast<uint32_t>(s->host.lights.size());
    o->bvh_width = s->host.width;
    o->build_seconds = s->build_seconds;
    o->stack_depth = s->host.stack_depth;
    return GR_OK;
}

gr_status gr_scene_last_stats(const gr_scene* s, gr_render_stats* o) {
    if (!s || !o) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    *o = s->stats;
    return GR_OK;
}

gr_status gr_film_create(uint32_t w, uint32_t h, gr_film** out) {
    if (!out || w == 0 || h == 0) return fail(GR_ERR_INVALID_ARGUMENT, "film size must be > 0");
    if (w > 32768 || h > 32768) return fail(GR_ERR_INVALID_ARGUMENT, "film size must be <= 32768");
    std::unique_ptr<gr_film> f(new gr_film());
    f->width = w;
    f->height = h;
    size_t bytes = static_cast<size_t>(w) * h * sizeof(float4);
    GR_CUDA_TRY(f->pixels.ensure(bytes));
    GR_CUDA_TRY(cudaMemset(f->pixels.ptr, 0, bytes));
    cudaGetDevice(&f->device);
    *out = f.release();
    return GR_OK;
}

gr_status gr_film_destroy(gr_film* f) {
    delete f;
    return GR_OK;
}

gr_status gr_film_clear(gr_film* f) {
    if (!f) return fail(GR_ERR_INVALID_ARGUMENT, "null film");
    GR_CUDA_TRY(cudaMemset(f->pixels.ptr, 0, static_cast<size_t>(f->width) * f->height * sizeof(float4)));
    if (f->splat.ptr) GR_CUDA_TRY(cudaMemset(f->splat.ptr, 0, static_cast<size_t>(f->width) * f->height * sizeof(float4)));
    f->passes = 0;
    return GR_OK;
}

static float splat_scale(const gr_film* f) { return f->passes ? 1.0f / static_cast<float>(f->passes) : 0.0f; }

gr_status gr_film_read_splat(const gr_film* f, float* splat) {
    if (!f || !splat) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    size_t n = static_cast<size_t>(f->width) * f->height;
    std::vector<float4> px(n, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    if (f->splat.ptr) GR_CUDA_TRY(cudaMemcpy(px.data(), f->splat.ptr, n * sizeof(float4), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i) {
        splat[3 * i] = px[i].x;
        splat[3 * i + 1] = px[i].y;
        splat[3 * i + 2] = px[i].z;
    }
    return GR_OK;
}

gr_status gr_film_read(const gr_film* f, float* accum, float* weight) {
    if (!f) return fail(GR_ERR_INVALID_ARGUMENT, "null film");
    if (!accum && !weight) return GR_OK;
    // The planes are split on the device and copied straight into the caller's arrays
    // (a DMA transfer when the caller's memory is pinned).
    const size_t n = static_cast<size_t>(f->width) * f->height;
    GR_CUDA_TRY(f->readback.ensure(n * 4 * sizeof(float)));
    float* acc_d = f->readback.as<float>();
    float* w_d = acc_d + 3 * n;
    GR_TRY(film_split(f->pixels.as<float4>(), static_cast<uint32_t>(n), acc_d, w_d, 0));
    if (accum) GR_CUDA_TRY(cudaMemcpyAsync(accum, acc_d, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, 0));
    if (weight) GR_CUDA_TRY(cudaMemcpyAsync(weight, w_d, n * sizeof(float), cudaMemcpyDeviceToHost, 0));
    GR_CUDA_TRY(cudaStreamSynchronize(0));
    return GR_OK;
}

gr_status gr_film_resolve(const gr_film* f, float* rgb) {
    if (!f || !rgb) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    uint32_t n = f->width * f->height;
    DevBuf out;
    GR_CUDA_TRY(out.ensure(static_cast<size_t>(n) * 3 * sizeof(float)));
    GR_TRY(film_resolve(f->pixels.as<float4>(), f->splat.as<float4>(), splat_scale(f), n, out.as<float>(), 0));
    GR_CUDA_TRY(cudaMemcpy(rgb, out.ptr, static_cast<size_t>(n) * 3 * sizeof(float), cudaMemcpyDeviceToHost));
    return GR_OK;
}

gr_status gr_film_write_exr(const gr_film* f, const char* path) {
    if (!f || !path) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    // Header and line-offset table (render/exr.rs:37-136) on the host, pixel data packed
    // on the device.
    std::vector<unsigned char> b;
    auto i32 = [&](int32_t v) {
        uint32_t u = static_cast<uint32_t>(v);
        for (int k = 0; k < 4; ++k) b.push_back(static_cast<unsigned char>((u >> (8 * k)) & 0xFF));
    };
    auto f32 = [&](float x) {
        int32_t u;
        std::memcpy(&u, &x, 4);
        i32(u);
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
    int32_t win[4] = {0, 0, static_cast<int32_t>(f->width) - 1, static_cast<int32_t>(f->height) - 1};
    for (const char* name : {"dataWindow", "displayWindow"}) {
        str(name);
        str("box2i");
        i32(16);
        for (int32_t v : win) i32(v);
    }
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
    f32(static_cast<float>(f->width));
    b.push_back(0);
    size_t line = 8 + static_cast<size_t>(f->width) * 12;
    size_t data_offset = b.size() + 8 * static_cast<size_t>(f->height);
    for (uint32_t y = 0; y < f->height; ++y) {
        uint64_t off = data_offset + y * line;
        for (int k = 0; k < 8; ++k) b.push_back(static_cast<unsigned char>((off >> (8 * k)) & 0xFF));
    }
    size_t data_bytes = line * f->height;
    DevBuf dev;
    GR_CUDA_TRY(dev.ensure(data_bytes));
    GR_TRY(film_exr_pack(f->pixels.as<float4>(), f->splat.as<float4>(), splat_scale(f), f->width, f->height,
                         dev.as<unsigned char>(), 0, 0));
    b.resize(data_offset + data_bytes);
    GR_CUDA_TRY(cudaMemcpy(b.data() + data_offset, dev.ptr, data_bytes, cudaMemcpyDeviceToHost));
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

static gr_status run_render(gr_scene* s, const gr_camera* c, const gr_render_params* p, uint32_t w, uint32_t h,
                            float4* film, float* samples_out, float4* splat = nullptr) {
    RenderJob job;
    job.scene = s->dev;
    job.camera = make_camera(*c);
    job.params = *p;
    job.width = w;
    job.height = h;
    job.film = film;
    job.splat = splat;
    job.samples_out = samples_out;
    cudaStream_t st = s->stream;
    std::memset(&s->stats, 0, sizeof(s->stats));
    GR_CUDA_TRY(s->counters.ensure(NUM_COUNTERS * sizeof(uint32_t)));
    GR_CUDA_TRY(cudaMemsetAsync(s->counters.ptr, 0, NUM_COUNTERS * sizeof(uint32_t), st));
    std::lock_guard<std::mutex> work_lock(device_work().mu);
    GR_CUDA_TRY(cudaEventRecord(s->ev0, st));
    gr_status r = p->integrator == GR_INTEGRATOR_BDPT ? render_bdpt(s, job, st) : render_pt(s, job, st);
    if (r != GR_OK) {
        cudaStreamSynchronize(st);
        return r;
    }
    GR_CUDA_TRY(cudaEventRecord(s->ev1, st));
    uint32_t cnt[NUM_COUNTERS];
    GR_CUDA_TRY(cudaMemcpyAsync(cnt, s->counters.ptr, sizeof(cnt), cudaMemcpyDeviceToHost, st));
    GR_CUDA_TRY(cudaStreamSynchronize(st));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->stats.device_ms = ms;
    uint64_t rays, shadow;
    std::memcpy(&rays, cnt + CNT_RAYS, 8);
    std::memcpy(&shadow, cnt + CNT_SHADOW, 8);
    s->stats.extension_rays = rays;
    s->stats.shadow_rays = shadow;
    std::memcpy(&s->stats.node_visits, cnt + CNT_NODES, 8);
    std::memcpy(&s->stats.prim_tests, cnt + CNT_PRIMS, 8);
    if (cnt[CNT_ERROR] == 2)
        return fail(GR_ERR_TIMEOUT, "traversal step budget exceeded (ray " + std::to_string(cnt[CNT_ERROR + 1]) + ")");
    if (cnt[CNT_ERROR] == 3) return fail(GR_ERR_TIMEOUT, "film accumulation: a wait between pass chunks ran out");
    if (cnt[CNT_ERROR]) return fail(GR_ERR_STACK_OVERFLOW, "traversal stack bound exceeded");
    return p->integrator == GR_INTEGRATOR_BDPT ? bdpt_index_check() : pt_index_check();
}

gr_status gr_render(gr_scene* s, const gr_camera* c, const gr_render_params* p, gr_film* f) {
    if (!s || !c || !f) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    GR_TRY(check_render_params(p));
    std::lock_guard<std::mutex> g(s->mu);
    float4* splat = nullptr;
    if (p->integrator == GR_INTEGRATOR_BDPT && p->light_tracing) {
        if (!f->splat.ptr) {
            size_t bytes = static_cast<size_t>(f->width) * f->height * sizeof(float4);
            GR_CUDA_TRY(f->splat.ensure(bytes));
            GR_CUDA_TRY(cudaMemset(f->splat.ptr, 0, bytes));
        }
        splat = f->splat.as<float4>();
    }
    GR_TRY(run_render(s, c, p, f->width, f->height, f->pixels.as<float4>(), nullptr, splat));
    f->passes += p->spp;
    return GR_OK;
}

gr_status gr_render_samples(gr_scene* s, const gr_camera* c, const gr_render_params* p, uint32_t w, uint32_t h,
                            float* out) {
    if (!s || !c || !out || w == 0 || h == 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
    GR_TRY(check_render_params(p));
    std::lock_guard<std::mutex> g(s->mu);
    size_t bytes = static_cast<size_t>(w) * h * 5 * sizeof(float);
    DevBuf dev;
    GR_CUDA_TRY(dev.ensure(bytes));
    GR_TRY(run_render(s, c, p, w, h, nullptr, dev.as<float>()));
    GR_CUDA_TRY(cudaMemcpy(out, dev.ptr, bytes, cudaMemcpyDeviceToHost));
    return GR_OK;
}

gr_status gr_trace_rays(gr_scene* s, const float* rays, uint64_t n, gr_hit* hits) {
    if (!s || (n && (!rays || !hits))) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    if (n == 0) return GR_OK;
    std::lock_guard<std::mutex> g(s->mu);
    Scratch sc;
    cudaError_t e;
    float* dr = static_cast<float*>(sc.get(n * 6 * sizeof(float), e));
    GR_CUDA_TRY(e);
    gr_hit* dh = static_cast<gr_hit*>(sc.get(n * sizeof(gr_hit), e));
    GR_CUDA_TRY(e);
    int* derr = static_cast<int*>(sc.get(sizeof(int), e));
    GR_CUDA_TRY(e);
    GR_CUDA_TRY(cudaMemsetAsync(derr, 0, sizeof(int), s->stream));
    GR_CUDA_TRY(cudaMemcpyAsync(dr, rays, n * 6 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    GR_TRY(launch_trace(s->dev, dr, n, dh, false, nullptr, derr, s->stream));
    GR_CUDA_TRY(cudaMemcpyAsync(hits, dh, n * sizeof(gr_hit), cudaMemcpyDeviceToHost, s->stream));
    int herr = 0;
    GR_CUDA_TRY(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    GR_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (herr == 2) return fail(GR_ERR_TIMEOUT, "traversal step budget exceeded");
    if (herr) return fail(GR_ERR_STACK_OVERFLOW, "traversal stack bound exceeded");
    return GR_OK;
}

gr_status gr_trace_rays_dev(gr_scene* s, const float* rays, uint64_t n, gr_hit* hits, void* stream) {
    if (!s || (n && (!rays || !hits))) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    GR_CUDA_TRY(s->counters.ensure(NUM_COUNTERS * sizeof(uint32_t)));
    int* err = reinterpret_cast<int*>(s->counters.as<uint32_t>() + CNT_ERROR);
    return launch_trace(s->dev, rays, n, hits, false, nullptr, err, static_cast<cudaStream_t>(stream));
}

gr_status gr_intersect_naive(gr_scene* s, const float* rays, uint64_t n, gr_hit* hits) {
    if (!s || (n && (!rays || !hits))) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    if (n == 0) return GR_OK;
    std::lock_guard<std::mutex> g(s->mu);
    Scratch sc;
    cudaError_t e;
    float* dr = static_cast<float*>(sc.get(n * 6 * sizeof(float), e));
    GR_CUDA_TRY(e);
    gr_hit* dh = static_cast<gr_hit*>(sc.get(n * sizeof(gr_hit), e));
    GR_CUDA_TRY(e);
    GR_CUDA_TRY(cudaMemcpyAsync(dr, rays, n * 6 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    GR_TRY(launch_naive(s->dev, dr, n, dh, s->stream));
    GR_CUDA_TRY(cudaMemcpyAsync(hits, dh, n * sizeof(gr_hit), cudaMemcpyDeviceToHost, s->stream));
    GR_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return GR_OK;
}

gr_status gr_visibility(gr_scene* s, const float* pairs, uint64_t n, uint8_t* visible) {
    if (!s || (n && (!pairs || !visible))) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    if (n == 0) return GR_OK;
    std::lock_guard<std::mutex> g(s->mu);
    Scratch sc;
    cudaError_t e;
    float* dp = static_cast<float*>(sc.get(n * 6 * sizeof(float), e));
    GR_CUDA_TRY(e);
    uint8_t* dv = static_cast<uint8_t*>(sc.get(n, e));
    GR_CUDA_TRY(e);
    int* derr = static_cast<int*>(sc.get(sizeof(int), e));
    GR_CUDA_TRY(e);
    GR_CUDA_TRY(cudaMemsetAsync(derr, 0, sizeof(int), s->stream));
    GR_CUDA_TRY(cudaMemcpyAsync(dp, pairs, n * 6 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    GR_TRY(launch_visibility(s->dev, dp, n, dv, derr, s->stream));
    GR_CUDA_TRY(cudaMemcpyAsync(visible, dv, n, cudaMemcpyDeviceToHost, s->stream));
    int herr = 0;
    GR_CUDA_TRY(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    GR_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (herr == 2) return fail(GR_ERR_TIMEOUT, "traversal step budget exceeded");
    if (herr) return fail(GR_ERR_STACK_OVERFLOW, "traversal stack bound exceeded");
    return GR_OK;
}

gr_status gr_sample_light(gr_scene* s, const float* u, uint64_t n, gr_light_sample* out) {
    if (!s || (n && (!u || !out))) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    if (s->dev.num_lights == 0) return fail(GR_ERR_INVALID_ARGUMENT, "scene has no lights");
    if (n == 0) return GR_OK;
    std::lock_guard<std::mutex> g(s->mu);
    Scratch sc;
    cudaError_t e;
    float* du = static_cast<float*>(sc.get(n * 6 * sizeof(float), e));
    GR_CUDA_TRY(e);
    gr_light_sample* dout = static_cast<gr_light_sample*>(sc.get(n * sizeof(gr_light_sample), e));
    GR_CUDA_TRY(e);
    GR_CUDA_TRY(cudaMemcpyAsync(du, u, n * 6 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    GR_TRY(launch_sample_light(s->dev, du, n, dout, s->stream));
    GR_CUDA_TRY(cudaMemcpyAsync(out, dout, n * sizeof(gr_light_sample), cudaMemcpyDeviceToHost, s->stream));
    GR_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return GR_OK;
}

static gr_status bsdf_call(int op, const gr_material_desc* md, uint64_t n, const gr_frame* fr, const float* wi,
                           const float* wo, const float* u, int32_t c2l, void* out, size_t out_bytes) {
    if (!md || (n && (!fr || !wi || !out))) return fail(GR_ERR_INVALID_ARGUMENT, "null argument");
    DevMaterial m;
    std::string err;
    if (!build_material(*md, m, err)) return fail(GR_ERR_INVALID_ARGUMENT, err);
    if (n == 0) return GR_OK;
    Scratch sc;
    cudaError_t e;
    DevMaterial* dm = static_cast<DevMaterial*>(sc.get(sizeof(DevMaterial), e));
    GR_CUDA_TRY(e);
    gr_frame* df = static_cast<gr_frame*>(sc.get(n * sizeof(gr_frame), e));
    GR_CUDA_TRY(e);
    float* dwi = static_cast<float*>(sc.get(n * 3 * sizeof(float), e));
    GR_CUDA_TRY(e);
    float* dwo = nullptr;
    float* du = nullptr;
    if (wo) {
        dwo = static_cast<float*>(sc.get(n * 3 * sizeof(float), e));
        GR_CUDA_TRY(e);
        GR_CUDA_TRY(cudaMemcpy(dwo, wo, n * 3 * sizeof(float), cudaMemcpyHostToDevice));
    }
    if (u) {
        du = static_cast<float*>(sc.get(n * 3 * sizeof(float), e));
        GR_CUDA_TRY(e);
        GR_CUDA_TRY(cudaMemcpy(du, u, n * 3 * sizeof(float), cudaMemcpyHostToDevice));
    }
    void* dout = sc.get(out_bytes, e);
    GR_CUDA_TRY(e);
    GR_CUDA_TRY(cudaMemcpy(dm, &m, sizeof(m), cudaMemcpyHostToDevice));
    GR_CUDA_TRY(cudaMemcpy(df, fr, n * sizeof(gr_frame), cudaMemcpyHostToDevice));
    GR_CUDA_TRY(cudaMemcpy(dwi, wi, n * 3 * sizeof(float), cudaMemcpyHostToDevice));
    GR_TRY(launch_bsdf(op, dm, n, df, dwi, dwo, du, c2l, dout, 0));
    GR_CUDA_TRY(cudaMemcpy(out, dout, out_bytes, cudaMemcpyDeviceToHost));
    return GR_OK;
}

gr_status gr_bsdf_eval(const gr_material_desc* m, uint64_t n, const gr_frame* fr, const float* in, const float* out,
                       int32_t c2l, float* f) {
    if (n && !out) return fail(GR_ERR_INVALID_ARGUMENT, "null outgoing");
    return bsdf_call(0, m, n, fr, in, out, nullptr, c2l, f, n * 3 * sizeof(float));
}

gr_status gr_bsdf_pdf(const gr_material_desc* m, uint64_t n, const gr_frame* fr, const float* in, const float* out,
                      float* pdf) {
    if (n && !out) return fail(GR_ERR_INVALID_ARGUMENT, "null outgoing");
    return bsdf_call(1, m, n, fr, in, out, nullptr, 0, pdf, n * sizeof(float));
}

gr_status gr_bsdf_sample_batch(const gr_material_desc* m, uint64_t n, const gr_frame* fr, const float* in,
                               const float* u, int32_t c2l, gr_bsdf_sample* o) {
    if (n && !u) return fail(GR_ERR_INVALID_ARGUMENT, "null uniforms");
    return bsdf_call(2, m, n, fr, in, nullptr, u, c2l, o, n * sizeof(gr_bsdf_sample));
}

gr_status gr_light_eval(const gr_material_desc* m, uint64_t n, const gr_frame* fr, const float* in, float* L) {
    return bsdf_call(3, m, n, fr, in, nullptr, nullptr, 0, L, n * 3 * sizeof(float));
}

}  // extern "C"
