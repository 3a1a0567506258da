// Wavefront unidirectional path tracer: PathTracerIntegrator::integrate
// (render/integrators.rs:42-100) and DisplayColorIntegrator (integrators.rs:18-34),
// driven as Stage::trace passes (render/stage.rs:23-36).
//
// Each camera path has a "slot" (pass-local sample index) holding its film position and,
// once it ends, its radiance; while it lives, its ray and state (throughput, radiance so
// far, random key) travel together in a compacted queue:
//   raygen   one slot per pixel and pass: jitter (film.rs:55-76), camera ray
//            (camera.rs:87-97), throughput 1, radiance 0
//   extend   closest hit for every queued ray (wide BVH, shared-memory stack)
//   shade    emission, Material::sample_world, throughput update, roulette and the
//            next ray; surviving paths are appended to the next queue with one
//            atomic per warp (ballot + popc)
//   film     after the last bounce, the deterministic tile gather in film.cu
// Extend and shade run as grid-stride loops over the device-side queue count, so the
// host never waits for a bounce; it polls the count two bounces behind to stop.
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "runtime.hpp"
#include "shade_sort.cuh"
#include "wavefront.cuh"

#define GR_TRY_S(expr)                \
    do {                              \
        gr_status s__ = (expr);       \
        if (s__ != GR_OK) return s__; \
    } while (0)

namespace gr {

namespace {

// Writes a group's starting queue length (the copy from a host variable it replaces
// would stage through pageable memory).
__global__ void k_set_count(uint32_t* c, uint32_t n) { *c = n; }

// Threads per block of the path tracer's shading kernel, each block sorting its chunk of
// the queue by code path.  With larger blocks, fewer blocks share an SM, so more of its
// warps run the same code path at a time; the register cap (85) and the warps per SM
// stay those of six 128-thread blocks.  On the 102,422-triangle 1024 x 1024 64-spp
// render, blocks of 128 / 384 / 768 measured 1585 / 1605 / 1726 Msamples/s (shading 37%
// / 36% / 31% of device time): one block per SM, whose warps all shade the same code
// path, relieves the instruction fetch that bounded the kernel.  A queue too short to
// give every SM two such blocks is shaded in 128-thread blocks instead, which spread
// it over all SMs.  One block of 1024 threads per SM (64 registers, some spilled) was
// slower than 768 (shading 9.38 vs 9.02 ms per render).
#ifndef GR_SHADE_BLOCK
#define GR_SHADE_BLOCK 768
#endif
constexpr int SHADE_BIG = GR_SHADE_BLOCK;
static_assert(SHADE_BIG == 128 || SHADE_BIG == 384 || SHADE_BIG == 768, "shading block of 128, 384 or 768 threads");
// Entries per thread per chunk: 64 at 128 threads, SHADE_BIG_PER at 768 (shade_sort.cuh).
template <int NT>
constexpr uint32_t shade_per() {
    return NT == 128 ? SHADE_PER_THREAD : (NT == 384 ? 96u : SHADE_BIG_PER);
}

struct PTParams {
    DevCamera cam;
    uint32_t width, height, npix;
    FastDiv by_npix, by_width;  // divisions by npix and width
    uint32_t first_pass;
    uint64_t seed;
    uint32_t max_depth, rr_depth, rr_aggr;
    uint32_t qcap;  // queue capacity (paths of the group)
};

// Path state travels with its ray in the queue, two float4 per queue entry:
//   state[2q]     = (throughput.xyz, radiance.x)
//   state[2q + 1] = (radiance.y, radiance.z, key low 32 bits, key high 32 bits)
// Shading reads it where the entry sits and writes it where the surviving path is pushed
// (consecutive positions per warp), instead of gathering and scattering slot-indexed
// arrays at random.  A finished path writes its radiance to its slot (the index of its
// film position), which the film gather reads.
//
// The first queue (camera rays) holds only rays: its entry q is path q (slot q), whose
// state is unit throughput, no radiance and the key of its pass and pixel, so shading
// makes that state instead of reading it; and their one origin (the pinhole's) is stored
// once, in q_o[0].  Raygen writes 24 bytes per path.
GR_D uint64_t state_key(float4 b) {
    return (static_cast<uint64_t>(__float_as_uint(b.w)) << 32) | __float_as_uint(b.z);
}

// The random key of path q of the group (pass first_pass + q / npix, pixel q % npix).
GR_D uint64_t first_key(const PTParams& p, uint32_t q) {
    const uint32_t pass_local = fast_div(q, p.by_npix);
    return path_key(p.seed, p.first_pass + pass_local, q - pass_local * p.npix);
}

__global__ void __launch_bounds__(BLOCK) k_raygen(PTParams p, uint32_t n, float2* __restrict__ st,
                                                  float4* __restrict__ q_o, float4* __restrict__ q_d) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t pass_local = fast_div(i, p.by_npix);
    uint32_t pixel = i - pass_local * p.npix;
    uint32_t row = fast_div(pixel, p.by_width);
    uint32_t col = pixel - row * p.width;
    uint64_t k = path_key(p.seed, p.first_pass + pass_local, pixel);
    float s, t;
    film_sample_point(p.width, p.height, row, col, k, s, t);
    V3 o, d;
    camera_ray(p.cam, s, t, o, d);
    st[i] = make_float2(s, t);
    if (i == 0) q_o[0] = make_float4(o.x, o.y, o.z, 0.0f);  // the pinhole origin, the same for every ray
    q_d[i] = make_float4(d.x, d.y, d.z, 0.0f);
}

// Appends this lane's surviving path (slot, ray, state) to the next queue with one atomic
// per warp (ballot + popc).  Every lane of the warp must call it.
GR_D void push_path(bool alive, uint32_t* count_out, uint32_t slot, V3 o, V3 d, float4 sa, float4 sb,
                    uint32_t* __restrict__ nslot, float4* __restrict__ no, float4* __restrict__ nd,
                    float4* __restrict__ nstate, uint32_t cap) {
    const unsigned lane = threadIdx.x & 31;
    unsigned m = __ballot_sync(0xffffffffu, alive);
    if (!m) return;
    int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == static_cast<unsigned>(leader)) base = atomicAdd(count_out, static_cast<uint32_t>(__popc(m)));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (alive) {
        uint32_t pos = base + __popc(m & ((1u << lane) - 1u));
        if (!GR_IN_RANGE(pos, cap)) return;
        nslot[pos] = slot;
        no[pos] = make_float4(o.x, o.y, o.z, 0.0f);
        nd[pos] = make_float4(d.x, d.y, d.z, 0.0f);
        nstate[2 * static_cast<size_t>(pos)] = sa;
        nstate[2 * static_cast<size_t>(pos) + 1] = sb;
    }
}

// Material-sorted shading (shade_sort.cuh): each block sorts its chunk of the queue by
// code path (chosen lobe type, the material's lobe types), then shades it in that order.

// FIRST: the queue of camera rays (no slots or states stored; see first_key).
template <int NT, bool FIRST>
__global__ void __launch_bounds__(NT, 768 / NT) k_shade(DeviceScene s, PTParams p, uint32_t depth,
                                                 const uint32_t* __restrict__ count_in,
                                                 const uint32_t* __restrict__ q_slot, const float4* __restrict__ q_o,
                                                 const float4* __restrict__ q_d, const float4* __restrict__ q_hit,
                                                 const float4* __restrict__ q_state, float4* __restrict__ L_buf,
                                                 uint32_t* count_out, uint32_t* __restrict__ nslot,
                                                 float4* __restrict__ no, float4* __restrict__ nd,
                                                 float4* __restrict__ nstate) {
    extern __shared__ unsigned char dsmem[];
    constexpr uint32_t PER = shade_per<NT>();
    const SortView sm = sort_view<NT, PER>(dsmem);
    const uint32_t n = *count_in;
    const uint32_t base = DIM_CAMERA_WALK + 4 * depth;
    // Block-uniform chunk loop (sort_chunk's barriers need every thread).
    const uint32_t per = chunk_per_thread<NT, PER>(n, gridDim.x);
    const uint32_t chunk = chunk_entries<NT>(n, gridDim.x, per);
    for (uint32_t c0 = blockIdx.x * chunk; c0 < n; c0 += gridDim.x * chunk) {
        const uint32_t cn = min(chunk, n - c0);
        sort_chunk<NT, PER>(sm, cn, per, [&](uint32_t i) {
            uint32_t q = c0 + i;
            const uint64_t key = FIRST ? first_key(p, q) : state_key(q_state[2 * q + 1]);
            return shade_bucket(s, __float_as_int(q_hit[q].y), uniform01(key, base), 0);
        });
        // Every lane runs every step so that all of them reach the ballot in push_path.
        for (uint32_t e = 0; e < per; ++e) {
            uint32_t i = e * NT + threadIdx.x;
            bool alive = false;
            uint32_t slot = 0;
            V3 new_o = v3zero(), new_d = v3zero();
            float4 sa = make_float4(0.0f, 0.0f, 0.0f, 0.0f), sb = sa;
            if (i < cn) {
                uint32_t q = c0 + sm.order[i];
                float4 h = q_hit[q];
                float4 o4 = q_o[FIRST ? 0u : q], d4 = q_d[q];  // camera rays share q_o[0]
                V3 o = V3{o4.x, o4.y, o4.z}, d = V3{d4.x, d4.y, d4.z};
                if (FIRST) {
                    slot = q;
                    const uint64_t k0 = first_key(p, q);
                    sa = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
                    sb = make_float4(0.0f, 0.0f, __uint_as_float(static_cast<uint32_t>(k0)),
                                     __uint_as_float(static_cast<uint32_t>(k0 >> 32)));
                } else {
                    slot = q_slot[q];
                    sa = q_state[2 * static_cast<size_t>(q)];
                    sb = q_state[2 * static_cast<size_t>(q) + 1];
                }
                V3 tp = V3{sa.x, sa.y, sa.z}, L = V3{sa.w, sb.x, sb.y};
                int32_t k = __float_as_int(h.y);
                if (k < 0) {
                    if (s.has_env) L = L + mul(tp, V3{s.env[0], s.env[1], s.env[2]});
                } else {
                    uint32_t prim;
                    Frame f = hit_frame(s, k, o, d, h.x, h.z, h.w, prim);
                    const DevMaterial& m = s.materials[__ldg(s.prim_material + prim)];
                    uint64_t key = state_key(sb);
                    MaterialSample ms = sample_world(m, -d, f, true, uniform01(key, base), uniform01(key, base + 1),
                                                     uniform01(key, base + 2));
                    L = L + mul(tp, ms.emission);
                    tp = mul(tp, ms.radiance * (fabsf(dot(f.normal, ms.outgoing)) / ms.pdf));
                    new_o = nudge(o + (d * h.x), ms.outgoing);
                    new_d = ms.outgoing;
                    if (depth > p.rr_depth || nearly_zero(tp)) {
                        float rv = uniform01(key, base + 3);
                        float lum = luminance(tp);
                        float prob =
                            depth > p.rr_aggr ? clamped_lerp(0.10f, 0.75f, lum) : clamped_lerp(0.25f, 1.00f, lum);
                        tp = rv < prob ? tp / prob : v3zero();
                    }
                    alive = !is_zero(tp) && (p.max_depth == 0 || depth + 1 < p.max_depth);
                }
                if (alive) {
                    sa = make_float4(tp.x, tp.y, tp.z, L.x);
                    sb = make_float4(L.y, L.z, sb.z, sb.w);
                } else {
                    L_buf[slot] = make_float4(L.x, L.y, L.z, 0.0f);
                }
            }
            push_path(alive, count_out, slot, new_o, new_d, sa, sb, nslot, no, nd, nstate, p.qcap);
        }
        __syncthreads();  // sm is reused by the next chunk
    }
}

// DisplayColorIntegrator: one bounce, so the queue is the camera rays (entry q is path q).
__global__ void __launch_bounds__(BLOCK) k_shade_display(DeviceScene s, const uint32_t* __restrict__ count_in,
                                                         const float4* __restrict__ q_hit, float4* __restrict__ L_buf) {
    const uint32_t n = *count_in;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        float4 h = q_hit[q];
        int32_t k = __float_as_int(h.y);
        float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (k >= 0) {
            uint32_t prim = __float_as_uint(__ldg(s.prims + 3 * static_cast<size_t>(k)).w);
            const DevMaterial& m = s.materials[__ldg(s.prim_material + prim)];
            c = make_float4(m.display[0], m.display[1], m.display[2], 0.0f);
        }
        L_buf[q] = c;
    }
}

template <int NT, bool FIRST, class... A>
gr_status launch_shade_nt(uint32_t n_bound, cudaStream_t st, A... a) {
    const size_t smem = sort_smem_bytes(NT, shade_per<NT>());
    GR_CUDA_TRY(allow_sort_smem(k_shade<NT, FIRST>, smem));
    // Every resident block; each picks its entries per thread from the queue length.
    int grid = resident_grid(k_shade<NT, FIRST>, smem, n_bound, NT);
    k_shade<NT, FIRST><<<grid, NT, smem, st>>>(a...);
    return GR_OK;
}

// Shades a queue of at most n_bound entries (the device holds the exact length): in
// SHADE_BIG-thread blocks while that fills two blocks per SM, else in 128-thread blocks.
// `first`: the queue of camera rays (depth 0).
template <class... A>
gr_status launch_shade(uint32_t n_bound, bool first, cudaStream_t st, A... a) {
    const bool big = SHADE_BIG != 128 && n_bound >= 2u * static_cast<uint32_t>(device_sm_count()) * SHADE_BIG;
    if (first) return big ? launch_shade_nt<SHADE_BIG, true>(n_bound, st, a...)
                          : launch_shade_nt<128, true>(n_bound, st, a...);
    return big ? launch_shade_nt<SHADE_BIG, false>(n_bound, st, a...) : launch_shade_nt<128, false>(n_bound, st, a...);
}

__global__ void k_samples_out(uint32_t n, const float2* __restrict__ st, const float4* __restrict__ L, float* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 a = st[i];
    float4 c = L[i];
    out[5 * i] = a.x;
    out[5 * i + 1] = a.y;
    out[5 * i + 2] = c.x;
    out[5 * i + 3] = c.y;
    out[5 * i + 4] = c.z;
}

uint32_t paths_in_flight_target() {
    const char* e = std::getenv("GR_PATHS_IN_FLIGHT");
    if (e && std::atoi(e) > 0) return static_cast<uint32_t>(std::atoi(e));
    // 64 M paths (about 9 GB): a 64-spp megapixel render is one group with one tail;
    // measured faster than 16 M (4 groups) and 32 M on that workload.
    return 1u << 26;
}

}  // namespace

cudaError_t PathState::ensure(size_t n) {
    if (n <= capacity && q_hit.ptr) return cudaSuccess;
    cudaError_t e;
#define GR_ENS(buf, bytes)                  \
    if ((e = (buf).ensure(bytes)) != cudaSuccess) return e;
    GR_ENS(light, n * sizeof(float4));
    GR_ENS(st, n * sizeof(float2));
    for (int k = 0; k < 2; ++k) {
        GR_ENS(q_slot[k], n * sizeof(uint32_t));
        GR_ENS(q_o[k], n * sizeof(float4));
        GR_ENS(q_d[k], n * sizeof(float4));
        GR_ENS(q_state[k], n * 2 * sizeof(float4));
    }
    GR_ENS(q_hit, n * sizeof(float4));
#undef GR_ENS
    capacity = n;
    return cudaSuccess;
}

gr_status render_pt(gr_scene* sc, const RenderJob& job, cudaStream_t st) {
    const gr_render_params& rp = job.params;
    const uint32_t npix = job.width * job.height;
    const bool display = rp.integrator == GR_INTEGRATOR_DISPLAY_COLOR;
    const uint32_t total = job.samples_out ? 1u : rp.spp;
    if (total == 0) return GR_OK;
    uint32_t group = std::max(1u, std::min(total, paths_in_flight_target() / std::max(1u, npix)));
    if (static_cast<uint64_t>(group) * npix > 0xFFFFFFFFull / 2) group = 1;
    PathState& ps = device_work().paths;
    GR_CUDA_TRY(ps.ensure(static_cast<size_t>(group) * npix));
    uint32_t* cnt = sc->counters.as<uint32_t>();
    int* err = reinterpret_cast<int*>(cnt + CNT_ERROR);
    unsigned long long* rays = reinterpret_cast<unsigned long long*>(cnt + CNT_RAYS);
    BounceReadback& rb = device_work().readback;  // the caller holds device_work().mu
    GR_CUDA_TRY(rb.ensure());
    uint32_t* host_cnt = rb.host;
    cudaEvent_t* evs = rb.ev;

    // Optional per-kernel timing: one event pair per extend / shade launch.
    const bool timed = (rp.flags & GR_RENDER_TIME_KERNELS) != 0;
    std::vector<cudaEvent_t> tev;
    struct FreeTev {
        std::vector<cudaEvent_t>& v;
        ~FreeTev() {
            for (cudaEvent_t e : v) cudaEventDestroy(e);
        }
    } free_tev{tev};
    std::vector<std::pair<int, int>> ext_pairs, shade_pairs, raygen_pairs, film_pairs;
    auto mark = [&](int& idx) -> gr_status {
        cudaEvent_t e;
        GR_CUDA_TRY(cudaEventCreate(&e));
        tev.push_back(e);
        idx = static_cast<int>(tev.size()) - 1;
        GR_CUDA_TRY(cudaEventRecord(e, st));
        return GR_OK;
    };

    PTParams p;
    p.cam = job.camera;
    p.width = job.width;
    p.by_width = make_fastdiv(job.width);
    p.height = job.height;
    p.npix = npix;
    p.by_npix = make_fastdiv(npix);
    p.qcap = static_cast<uint32_t>(static_cast<size_t>(group) * npix);
    p.seed = rp.seed;
    p.max_depth = display ? 1 : rp.max_depth;
    p.rr_depth = rp.rr_depth;
    p.rr_aggr = rp.rr_aggressive_depth;
    uint64_t launches = 0;

    for (uint32_t done = 0; done < total; done += group) {
        uint32_t g = std::min(group, total - done);
        uint32_t n = g * npix;
        p.first_pass = rp.first_pass + done;
        int r0 = -1, r1 = -1;
        if (timed) GR_TRY_S(mark(r0));
        k_set_count<<<1, 1, 0, st>>>(cnt + CNT_QUEUE0, n);
        GR_CUDA_TRY(cudaGetLastError());
        uint32_t bound = n;  // an upper bound of the current queue length
        k_raygen<<<(n + BLOCK - 1) / BLOCK, BLOCK, 0, st>>>(p, n, ps.st.as<float2>(), ps.q_o[0].as<float4>(),
                                                            ps.q_d[0].as<float4>());
        GR_CUDA_TRY(cudaGetLastError());
        ++launches;
        GR_TRY_S(sync_check(st, "raygen", 0, n));
        if (timed) {
            GR_TRY_S(mark(r1));
            raygen_pairs.emplace_back(r0, r1);
        }
        for (uint32_t depth = 0;; ++depth) {
            if (p.max_depth && depth >= p.max_depth) break;
            int cur = depth & 1, nxt = cur ^ 1;
            int e0 = -1, e1 = -1;
            if (timed) GR_TRY_S(mark(e0));
            gr_status s1 = extend_any(job.scene, (rp.flags & GR_RENDER_COUNT_TRAVERSAL) != 0, n, cnt + cur,
                                      ps.q_o[cur].as<float4>(), ps.q_d[cur].as<float4>(), ps.q_hit.as<float4>(), err,
                                      rays, cnt + CNT_FETCH, st, depth == 0);
            if (s1 != GR_OK) return s1;
            GR_CUDA_TRY(cudaGetLastError());
            ++launches;
            GR_TRY_S(sync_check(st, "extend", depth, n));
            if (timed) {
                GR_TRY_S(mark(e1));
                ext_pairs.emplace_back(e0, e1);
            }
            if (display) {
                int grid = resident_grid(k_shade_display, 0, n);
                k_shade_display<<<grid, BLOCK, 0, st>>>(job.scene, cnt + cur, ps.q_hit.as<float4>(),
                                                        ps.light.as<float4>());
                GR_CUDA_TRY(cudaGetLastError());
                ++launches;
                break;
            }
            GR_CUDA_TRY(cudaMemsetAsync(cnt + nxt, 0, sizeof(uint32_t), st));
            if (timed) GR_TRY_S(mark(e0));
            GR_TRY_S(launch_shade(bound, depth == 0, st, job.scene, p, depth, cnt + cur, ps.q_slot[cur].as<uint32_t>(),
                                  ps.q_o[cur].as<float4>(), ps.q_d[cur].as<float4>(), ps.q_hit.as<float4>(),
                                  ps.q_state[cur].as<float4>(), ps.light.as<float4>(), cnt + nxt,
                                  ps.q_slot[nxt].as<uint32_t>(), ps.q_o[nxt].as<float4>(), ps.q_d[nxt].as<float4>(),
                                  ps.q_state[nxt].as<float4>()));
            GR_CUDA_TRY(cudaGetLastError());
            ++launches;
            GR_TRY_S(sync_check(st, "shade", depth, n));
            if (timed) {
                GR_TRY_S(mark(e1));
                shade_pairs.emplace_back(e0, e1);
            }
            GR_CUDA_TRY(cudaMemcpyAsync(host_cnt + (depth & 3), cnt + nxt, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                        st));
            GR_CUDA_TRY(cudaEventRecord(evs[depth & 3], st));
            if (depth >= 2) {
                GR_CUDA_TRY(cudaEventSynchronize(evs[(depth - 2) & 3]));
                if (host_cnt[(depth - 2) & 3] == 0) break;
                // Paths only leave the queue within a group, so the length known for
                // bounce depth - 1 bounds every later bounce's.
                bound = host_cnt[(depth - 2) & 3];
            }
        }
        if (job.film) {
            int f0 = -1, f1 = -1;
            if (timed) GR_TRY_S(mark(f0));
            DevBuf& fs = device_work().film_sched;
            GR_CUDA_TRY(fs.ensure(film_sched_words(job.width, job.height) * sizeof(uint32_t)));
            gr_status s2 = film_gather(ps.st.as<float2>(), ps.light.as<float4>(), job.width, job.height, g, job.film,
                                       st, fs.as<uint32_t>(), err);
            if (s2 != GR_OK) return s2;
            ++launches;
            if (timed) {
                GR_TRY_S(mark(f1));
                film_pairs.emplace_back(f0, f1);
            }
        }
        if (job.samples_out) {
            k_samples_out<<<(n + 255) / 256, 256, 0, st>>>(n, ps.st.as<float2>(), ps.light.as<float4>(),
                                                          job.samples_out);
            GR_CUDA_TRY(cudaGetLastError());
            ++launches;
        }
    }
    sc->stats.samples += static_cast<uint64_t>(total) * npix;
    sc->stats.kernel_launches += launches;
    if (timed) {
        GR_CUDA_TRY(cudaStreamSynchronize(st));
        auto sum = [&](const std::vector<std::pair<int, int>>& pairs, double& out) -> gr_status {
            for (auto& pr : pairs) {
                float ms = 0.0f;
                GR_CUDA_TRY(cudaEventElapsedTime(&ms, tev[pr.first], tev[pr.second]));
                out += ms;
            }
            return GR_OK;
        };
        GR_TRY_S(sum(ext_pairs, sc->stats.extend_ms));
        GR_TRY_S(sum(shade_pairs, sc->stats.shade_ms));
        GR_TRY_S(sum(raygen_pairs, sc->stats.raygen_ms));
        GR_TRY_S(sum(film_pairs, sc->stats.film_ms));
        sc->stats.extend_launches += ext_pairs.size();
    }
    return GR_OK;
}

int device_sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace gr

// ---------------------------------------------------------------------------
// Render entry point that allocates nothing.
//
// Some callers cannot let a library allocate device memory: an application that owns
// all GPU memory through its own pool and forbids hidden allocations (a host program
// that embeds this renderer under a fixed memory budget), or a real-time frame loop
// that a cudaMalloc / cudaFree would stall, since both synchronise the whole device.
// For them, gr_render_static runs the same wavefront kernels as gr_render, with the
// path state and queues in one fixed device array of this library instead of buffers
// of the scene.  The caller passes the inputs (scene, camera, settings) and the output
// (a device film of width * height float4 {accum.rgb, weight}, accumulated into).
//
// Limits and sharing:
//   - at most STATIC_MAX_PATHS (131072) pixels per image; larger sizes are rejected;
//   - the array (STATIC_SCRATCH_BYTES, about 23 MB) is held by every GPU that loads the
//     library until the process exits;
//   - every call uses the same array and it keeps the last call's contents (each call
//     clears the counters it needs), so calls that overlap on the GPU (other threads,
//     other streams) race: serialise them;
//   - the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call before any
//     stream capture;
//   - the call returns once its work on the stream has finished: it waits for the
//     stream at the end to read the traversal status (GR_ERR_TIMEOUT,
//     GR_ERR_STACK_OVERFLOW, as gr_render reports them), and with max_depth == 0 (the
//     reference's unbounded depth) also every 4 bounces to see whether any path is left.
namespace gr {
namespace {

constexpr uint32_t STATIC_MAX_PATHS = 1u << 17;
// Per path: light (float4), st (float2), queue slot x2, queue o/d x2 (float4), queue
// state x2 (2 float4), hit (float4); plus a 256-byte block of counters.
constexpr size_t STATIC_PER_PATH = 16 + 8 + 2 * 4 + 2 * 16 + 2 * 16 + 2 * 32 + 16;
constexpr size_t STATIC_SCRATCH_BYTES = STATIC_MAX_PATHS * STATIC_PER_PATH + 256;

static __device__ __align__(256) unsigned char g_static_scratch[STATIC_SCRATCH_BYTES];

constexpr int STATIC_MAX_DEVICES = 64;
std::mutex g_static_mu;
void* g_static_ptr[STATIC_MAX_DEVICES] = {nullptr};

// Device address of g_static_scratch for the current device, looked up once.
gr_status static_scratch(void** out) {
    int dev = 0;
    GR_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= STATIC_MAX_DEVICES) {
        set_error("device index out of range for the static scratch table");
        return GR_ERR_INTERNAL;
    }
    std::lock_guard<std::mutex> g(g_static_mu);
    if (!g_static_ptr[dev]) {
        void* p = nullptr;
        GR_CUDA_TRY(cudaGetSymbolAddress(&p, g_static_scratch));
        g_static_ptr[dev] = p;
    }
    *out = g_static_ptr[dev];
    return GR_OK;
}

}  // namespace

gr_status pt_index_check() {
#if GR_CHECKED
    bool bad = false;
    GR_CUDA_TRY(take_bad_index(bad));
    if (bad) {
        set_error("path tracer: a queue or entry index was out of range (checked build)");
        return GR_ERR_INTERNAL;
    }
#endif
    return GR_OK;
}

}  // namespace gr

using namespace gr;

extern "C" gr_status gr_render_static(gr_scene* sc, const gr_camera* camera, const gr_render_params* rp,
                                      uint32_t width, uint32_t height, float* film_dev, void* stream) {
    if (!sc || !camera || !rp || !film_dev || width == 0 || height == 0) {
        set_error("gr_render_static: null argument or empty image");
        return GR_ERR_INVALID_ARGUMENT;
    }
    GR_TRY_S(check_render_params(rp));
    if (rp->integrator != GR_INTEGRATOR_PATH_TRACER && rp->integrator != GR_INTEGRATOR_DISPLAY_COLOR) {
        set_error("gr_render_static: only the path tracer and the display-colour integrator are supported");
        return GR_ERR_UNSUPPORTED;
    }
    const uint64_t npix64 = static_cast<uint64_t>(width) * height;
    if (npix64 > STATIC_MAX_PATHS) {
        set_error("gr_render_static: width * height = " + std::to_string(npix64) + " exceeds the fixed maximum of " +
                  std::to_string(STATIC_MAX_PATHS) + " pixels");
        return GR_ERR_INVALID_ARGUMENT;
    }
    if (rp->spp == 0) return GR_OK;
    // Held for the whole call, which ends after its device work: gr_scene_destroy on
    // another thread waits for it.
    std::lock_guard<std::mutex> scene_lock(sc->mu);
    void* base = nullptr;
    GR_TRY_S(static_scratch(&base));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint32_t npix = static_cast<uint32_t>(npix64);
    const size_t cap = STATIC_MAX_PATHS;
    // Carve the array (same layout for every call; every region is 16-byte aligned).
    unsigned char* b = static_cast<unsigned char*>(base);
    uint32_t* cnt = reinterpret_cast<uint32_t*>(b);
    size_t off = 256;
    auto take = [&](size_t bytes) {
        void* p = b + off;
        off += bytes;
        return p;
    };
    float4* light = static_cast<float4*>(take(cap * sizeof(float4)));
    float4* q_state[2];
    q_state[0] = static_cast<float4*>(take(cap * 2 * sizeof(float4)));
    q_state[1] = static_cast<float4*>(take(cap * 2 * sizeof(float4)));
    float2* stb = static_cast<float2*>(take(cap * sizeof(float2)));
    float4* q_o[2];
    float4* q_d[2];
    q_o[0] = static_cast<float4*>(take(cap * sizeof(float4)));
    q_o[1] = static_cast<float4*>(take(cap * sizeof(float4)));
    q_d[0] = static_cast<float4*>(take(cap * sizeof(float4)));
    q_d[1] = static_cast<float4*>(take(cap * sizeof(float4)));
    float4* q_hit = static_cast<float4*>(take(cap * sizeof(float4)));
    uint32_t* q_slot[2];
    q_slot[0] = static_cast<uint32_t*>(take(cap * sizeof(uint32_t)));
    q_slot[1] = static_cast<uint32_t*>(take(cap * sizeof(uint32_t)));
    int* err = reinterpret_cast<int*>(cnt + CNT_ERROR);
    unsigned long long* rays = reinterpret_cast<unsigned long long*>(cnt + CNT_RAYS);

    const bool display = rp->integrator == GR_INTEGRATOR_DISPLAY_COLOR;
    PTParams p;
    p.cam = make_camera(*camera);
    p.width = width;
    p.by_width = make_fastdiv(width);
    p.height = height;
    p.npix = npix;
    p.by_npix = make_fastdiv(npix);
    p.qcap = npix;
    p.seed = rp->seed;
    p.max_depth = display ? 1 : rp->max_depth;
    p.rr_depth = rp->rr_depth;
    p.rr_aggr = rp->rr_aggressive_depth;
    // The array keeps the previous call's contents: clear the counters every call.
    GR_CUDA_TRY(cudaMemsetAsync(cnt, 0, 256, st));
    for (uint32_t pass = 0; pass < rp->spp; ++pass) {
        p.first_pass = rp->first_pass + pass;
        uint32_t n = npix;
        k_set_count<<<1, 1, 0, st>>>(cnt + CNT_QUEUE0, n);
        k_raygen<<<(n + BLOCK - 1) / BLOCK, BLOCK, 0, st>>>(p, n, stb, q_o[0], q_d[0]);
        GR_CUDA_TRY(cudaGetLastError());
        for (uint32_t depth = 0;; ++depth) {
            if (p.max_depth && depth >= p.max_depth) break;
            int cur = depth & 1, nxt = cur ^ 1;
            GR_TRY_S(extend_any(sc->dev, false, n, cnt + cur, q_o[cur], q_d[cur], q_hit, err, rays, cnt + CNT_FETCH,
                                st, depth == 0));
            GR_CUDA_TRY(cudaGetLastError());
            if (display) {
                int grid = resident_grid(k_shade_display, 0, n);
                k_shade_display<<<grid, BLOCK, 0, st>>>(sc->dev, cnt + cur, q_hit, light);
                GR_CUDA_TRY(cudaGetLastError());
                break;
            }
            GR_CUDA_TRY(cudaMemsetAsync(cnt + nxt, 0, sizeof(uint32_t), st));
            GR_TRY_S(launch_shade(n, depth == 0, st, sc->dev, p, depth, cnt + cur, q_slot[cur], q_o[cur], q_d[cur], q_hit,
                                  q_state[cur], light, cnt + nxt, q_slot[nxt], q_o[nxt], q_d[nxt], q_state[nxt]));
            GR_CUDA_TRY(cudaGetLastError());
            if (p.max_depth == 0 && (depth & 3) == 3) {
                // Unbounded (reference) depth: stop once no path is left.  The copy goes
                // to a stack variable; no host or device memory is allocated.
                uint32_t left = 0;
                GR_CUDA_TRY(cudaMemcpyAsync(&left, cnt + nxt, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
                GR_CUDA_TRY(cudaStreamSynchronize(st));
                if (left == 0) break;
            }
        }
        GR_TRY_S(film_gather(stb, light, width, height, 1, reinterpret_cast<float4*>(film_dev), st));
    }
    // The traversal status of every pass, read like gr_render reads it: a ray over the
    // step budget (2) or the stack bound (1), and the ray index.
    int status[2] = {0, 0};
    GR_CUDA_TRY(cudaMemcpyAsync(status, err, sizeof(status), cudaMemcpyDeviceToHost, st));
    GR_CUDA_TRY(cudaStreamSynchronize(st));
    if (status[0] == 2) {
        set_error("gr_render_static: traversal step budget exceeded (ray " + std::to_string(status[1]) + ")");
        return GR_ERR_TIMEOUT;
    }
    if (status[0]) {
        set_error("gr_render_static: traversal stack bound exceeded");
        return GR_ERR_STACK_OVERFLOW;
    }
    return pt_index_check();
}
