// Host objects behind the C ABI handles, device buffers and the launch interface
// between the C ABI (api.cu) and the kernel files.
#pragma once

#include <atomic>
#include <cstdlib>

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "scene.hpp"
#include "shading.cuh"

namespace gr {

void set_error(const std::string& msg);

#define GR_CUDA_TRY(expr)                                                                          \
    do {                                                                                           \
        cudaError_t e__ = (expr);                                                                  \
        if (e__ != cudaSuccess) {                                                                  \
            ::gr::set_error(std::string(#expr) + ": " + cudaGetErrorString(e__));                  \
            return e__ == cudaErrorMemoryAllocation ? GR_ERR_OUT_OF_MEMORY : GR_ERR_CUDA;          \
        }                                                                                          \
    } while (0)

// A device allocation that frees itself.
// Host-side fault injection for tests (no GPU fault): GR_FAIL_ALLOC_AT=k makes the k-th
// device allocation of the process report cudaErrorMemoryAllocation, once.
inline bool alloc_should_fail() {
    static const long at = [] {
        const char* e = std::getenv("GR_FAIL_ALLOC_AT");
        return e ? std::atol(e) : 0L;
    }();
    if (at <= 0) return false;
    static std::atomic<long> count{0};
    return count.fetch_add(1) + 1 == at;
}

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    DevBuf() {}
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t n) {
        if (n <= bytes) return cudaSuccess;
        release();
        if (alloc_should_fail()) return cudaErrorMemoryAllocation;
        cudaError_t e = cudaMalloc(&ptr, n);
        if (e == cudaSuccess) bytes = n;
        else ptr = nullptr;
        return e;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(ptr);
    }
};

// Path-tracer wavefront state, reused across renders of a scene (grown on demand).
struct PathState {
    DevBuf light, st;  // per slot: final radiance, film (s, t)
    // Ping-pong queues of live paths: slot, ray, and state (throughput, radiance so far,
    // random key: two float4 per entry); one hit per entry.  The first queue of a group
    // (camera rays) holds rays only: entry q is path q, whose state shading makes.
    DevBuf q_slot[2], q_o[2], q_d[2], q_state[2], q_hit;
    size_t capacity = 0;
    cudaError_t ensure(size_t n);
};

// BDPT walk queues, vertex storage, strategy entries and the shadow queue (grown on
// demand).  Walks are addressed by slot (2 per path: camera, light).
struct BdptState {
    DevBuf q_slot[2], q_o[2], q_d[2], q_hit, tp, key, st, light;
    DevBuf verts, vcount, flags, escape, entry_base, entries, shadow, lt, lt_pixel;
    DevBuf order, len_hist;  // paths ordered by walk lengths for the connection kernel
    cudaError_t ensure(size_t paths, uint32_t max_len);
    static size_t bytes_per_path(uint32_t max_len);  // device bytes ensure() needs per path
};

// The large wavefront buffers are shared by every scene on a device (renders on one
// GPU run one after another anyway); a scene keeps only its small counter block.
// The path tracer's view of its queue lengths: a pinned copy of the last four bounces'
// counts and an event after each copy.  Made once per device and kept (freeing pinned
// memory synchronises the device), so a render starts without host allocations.
struct BounceReadback {
    uint32_t* host = nullptr;
    cudaEvent_t ev[4] = {};
    cudaError_t ensure() {
        if (host) return cudaSuccess;
        for (cudaEvent_t& e : ev) {
            if (e) continue;
            cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
            if (r != cudaSuccess) return r;
        }
        return cudaHostAlloc(reinterpret_cast<void**>(&host), 4 * sizeof(uint32_t), cudaHostAllocDefault);
    }
};

struct DeviceWork {
    std::mutex mu;
    PathState paths;
    BdptState bdpt;
    BounceReadback readback;
    DevBuf film_sched;  // film_gather's chunk counter and tile flags
};
DeviceWork& device_work();  // of the current device

constexpr int CNT_QUEUE0 = 0;
constexpr int CNT_QUEUE1 = 1;
constexpr int CNT_ERROR = 2;
constexpr int CNT_RAYS = 4;    // 64-bit counter at index 4..5
constexpr int CNT_SHADOW = 6;  // 64-bit counter at index 6..7
constexpr int CNT_NODES = 8;   // 64-bit: BVH nodes visited (GR_RENDER_COUNT_TRAVERSAL)
constexpr int CNT_PRIMS = 10;  // 64-bit: primitives tested
constexpr int CNT_FETCH = 12;  // rays handed out by the refilling extension kernel (per launch)
constexpr int NUM_COUNTERS = 16;

struct SceneBuffers {
    DevBuf nodes, prims, tri_nidx, tri_uvidx, normals, uvs, prim_material, materials, lights, light_tris,
        light_nidx, light_uvidx, light_cdf;
};

}  // namespace gr

struct gr_scene {
    gr::HostBuild host;
    gr::SceneBuffers buf;
    gr::DeviceScene dev{};
    gr::DevBuf counters;  // [0..1] queue counts, [2] error flag, [3..] stats (gr::CNT_*)
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    gr_render_stats stats{};
    double build_seconds = 0.0;
    uint64_t device_bytes = 0;
    std::mutex mu;
    // Server requests that hold the scene (gr::scene_retain); gr_scene_destroy of a held
    // scene only marks it, and the last gr::scene_release frees it.  Both fields are
    // guarded by one library-wide mutex.
    uint32_t holders = 0;
    bool destroy_pending = false;
};

struct gr_film {
    uint32_t width = 0, height = 0;
    gr::DevBuf pixels;  // float4 (accum.rgb, weight) per pixel
    gr::DevBuf splat;   // float4 light-tracing splat sums (BDPT extension); allocated on first use
    mutable gr::DevBuf readback;  // accum and weight planes for gr_film_read (a cache); allocated on first use
    uint32_t passes = 0;
    int device = 0;
};

namespace gr {

// Device BVH build (bvh_build.cu) for a HostBuild made with GR_BUILD_DEVICE_LBVH:
// fills b.nodes, b.prims, b.tri_nidx, b.tri_uvidx (leaf order).
gr_status build_bvh_device(const HostBuild& h, SceneBuffers& b, cudaStream_t st, uint32_t& num_wide,
                           uint32_t& stack_depth, uint64_t& bytes);

// Kernel-side entry points (implemented in the .cu files).
gr_status launch_trace(const DeviceScene& s, const float* rays, uint64_t n, gr_hit* hits, bool any_hit,
                       const float* tmax, int* err, cudaStream_t st);
gr_status launch_naive(const DeviceScene& s, const float* rays, uint64_t n, gr_hit* hits, cudaStream_t st);
gr_status launch_visibility(const DeviceScene& s, const float* pairs, uint64_t n, uint8_t* vis, int* err,
                            cudaStream_t st);
gr_status launch_sample_light(const DeviceScene& s, const float* u, uint64_t n, gr_light_sample* out,
                              cudaStream_t st);
gr_status launch_bsdf(int op, const DevMaterial* m, uint64_t n, const gr_frame* frames, const float* wi,
                      const float* wo, const float* u, int c2l, void* out, cudaStream_t st);

struct RenderJob {
    DeviceScene scene;
    DevCamera camera;
    gr_render_params params;
    uint32_t width, height;
    float4* film;  // accumulate target, or null (samples only)
    float4* splat = nullptr;  // light-tracing splat target (BDPT extension), or null
    float* samples_out;  // device (s, t, r, g, b) per pixel for gr_render_samples, or null
};

gr_status render_pt(gr_scene* sc, const RenderJob& job, cudaStream_t st);
gr_status render_bdpt(gr_scene* sc, const RenderJob& job, cudaStream_t st);
// Checked builds (GR_CHECKED): whether a render's kernels wrote out of range (read after
// the render's work has finished); GR_OK otherwise.
// Scene lifetime across server requests: a request retains its scene from submission
// until no queued path can reach it any more; gr_scene_destroy waits for the last release.
void scene_retain(gr_scene* s);
void scene_release(gr_scene* s);

gr_status pt_index_check();
gr_status bdpt_index_check();
// Adds `passes` passes of samples (pass k at k * width * height in st_buf and color) to
// `film`, each pixel's sum in the reference's serial order.  With `sched` (device
// scratch of film_sched_words(width, height) words) and `err` (the error word; 3 = a
// wait between chunks ran out), many passes over a large image run as ordered chunks of
// passes (film.cu); otherwise one block per tile.
gr_status film_gather(const float2* st_buf, const float4* color, uint32_t width, uint32_t height, uint32_t passes,
                      float4* film, cudaStream_t s, uint32_t* sched = nullptr, int* err = nullptr);
size_t film_sched_words(uint32_t width, uint32_t height);
// Resolve and EXR packing add splat * splat_scale when splat is not null.
gr_status film_resolve(const float4* film, const float4* splat, float splat_scale, uint32_t n, float* rgb,
                       cudaStream_t s);
// Splits the float4 film into an accum plane (3 floats per pixel) and a weight plane.
gr_status film_split(const float4* film, uint32_t n, float* accum, float* weight, cudaStream_t s);
gr_status film_exr_pack(const float4* film, const float4* splat, float splat_scale, uint32_t width, uint32_t height,
                        unsigned char* out, size_t data_offset, cudaStream_t s);

int device_sm_count();

// Bounded host wait (GR_SYNC_CHECK=<seconds> in the environment; 0 = off): after a
// launch, polls the stream until it drains or the deadline passes.  On a timeout it
// records which kernel and bounce did not finish and returns GR_ERR_TIMEOUT, so a stuck
// kernel is reported instead of blocking the caller forever.
gr_status sync_check(cudaStream_t st, const char* what, uint32_t bounce, uint32_t n);

// Validates a gr_render_params (integrator kind, BDPT depth, extensions that apply to
// BDPT only); sets the error text and returns GR_ERR_INVALID_ARGUMENT when it fails.
gr_status check_render_params(const gr_render_params* p);

// Camera::new (core/camera.rs:42-61) evaluated on the host.
DevCamera make_camera(const gr_camera& c);

}  // namespace gr
