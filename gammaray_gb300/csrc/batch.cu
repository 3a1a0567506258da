// Batched rendering and the serving loop over the multi-job engine (engine.hpp).
// Neither has a counterpart in the reference, which renders one image per
// Stage::trace call (render/stage.rs:23-36).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "engine.hpp"

using namespace gr;

namespace {

thread_local gr_render_stats g_batch_stats{};

// Engines are costly to set up (up to a few GB of buffers and a captured graph), so the
// most recently used ones are kept, per configuration, and reset between batches.
constexpr size_t ENGINE_CACHE_MAX = 2;
std::mutex g_cache_mu;
using EngineKey = std::tuple<int, uint32_t, uint32_t, uint32_t>;
std::map<EngineKey, std::unique_ptr<Engine>> g_cache;
std::map<EngineKey, uint64_t> g_cache_used;  // last use, for eviction
uint64_t g_cache_clock = 0;

gr_status cached_engine(const EngineConfig& cfg, Engine*& out) {
    int dev = 0;
    GR_CUDA_TRY(cudaGetDevice(&dev));
    auto key = std::make_tuple(dev, cfg.capacity, cfg.width, cfg.block);
    auto it = g_cache.find(key);
    if (it == g_cache.end()) {
        while (g_cache.size() >= ENGINE_CACHE_MAX) {  // evict the least recently used
            auto lru = g_cache_used.begin();
            for (auto u = g_cache_used.begin(); u != g_cache_used.end(); ++u)
                if (u->second < lru->second) lru = u;
            g_cache.erase(lru->first);
            g_cache_used.erase(lru);
        }
        std::unique_ptr<Engine> e(new Engine());
        gr_status s = e->init(cfg, nullptr);
        if (s != GR_OK) return s;
        it = g_cache.emplace(key, std::move(e)).first;
    } else {
        gr_status s = it->second->reset();
        if (s != GR_OK) return s;
    }
    g_cache_used[key] = ++g_cache_clock;
    out = it->second.get();
    return GR_OK;
}

gr_status check_job(const gr_job& j) {
    if (!j.scene || !j.film) {
        set_error("batch job with a null scene or film");
        return GR_ERR_INVALID_ARGUMENT;
    }
    if (j.params.integrator < 0 || j.params.integrator > 2) {
        set_error("batch job with an unknown integrator");
        return GR_ERR_INVALID_ARGUMENT;
    }
    return GR_OK;
}

// Runs PT / display-colour jobs of one BVH width through one engine; units are issued
// round-robin over jobs, pass by pass.
gr_status run_engine_batch(const std::vector<const gr_job*>& jobs, const EngineConfig& cfg, gr_render_stats& st,
                           float4* const* films_override) {
    Engine* e = nullptr;
    gr_status s = cached_engine(cfg, e);
    if (s != GR_OK) return s;
    uint32_t max_spp = 0;
    std::vector<uint32_t> idx(jobs.size());
    for (size_t k = 0; k < jobs.size(); ++k) {
        const gr_job& j = *jobs[k];
        float4* film = films_override ? films_override[k] : j.film->pixels.as<float4>();
        DevJob dj = make_job(j.scene, j.camera, j.params, j.film->width, j.film->height, film);
        s = e->add_job(dj, 0, 0, idx[k]);
        if (s != GR_OK) return s;
        max_spp = std::max(max_spp, j.params.spp);
    }
    // Job-major order: a few scenes are live at a time, so their BVHs stay in L2; the
    // pool still refills across job boundaries.
    std::vector<std::pair<uint32_t, uint32_t>> units;
    for (size_t k = 0; k < jobs.size(); ++k)
        for (uint32_t r = 0; r < jobs[k]->params.spp; ++r) units.emplace_back(idx[k], jobs[k]->params.first_pass + r);
    (void)max_spp;
    s = e->append_units(units);
    if (s != GR_OK) return s;
    cudaEvent_t a, b;
    GR_CUDA_TRY(cudaEventCreate(&a));
    GR_CUDA_TRY(cudaEventCreate(&b));
    GR_CUDA_TRY(cudaEventRecord(a, e->stream()));
    bool done = false;
    s = e->run(0xFFFFFFFFu, done);
    GR_CUDA_TRY(cudaEventRecord(b, e->stream()));
    GR_CUDA_TRY(cudaEventSynchronize(b));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (s != GR_OK) return s;
    EngineCtl c;
    s = e->read_ctl(c);
    if (s != GR_OK) return s;
    st.samples += c.paths_total;  // all finished: the batch ran to completion
    st.extension_rays += c.rays;
    st.kernel_launches += static_cast<uint64_t>(c.iter) * 6;
    st.device_ms += ms;
    if (!done) {
        set_error("batch did not complete");
        return GR_ERR_INTERNAL;
    }
    return GR_OK;
}

// The options' capacity, else one sized from the batch: the smallest power of two that
// holds all its samples, between 1 M and 64 M paths (larger capacities amortise the
// per-iteration launches; small batches keep their buffers small).
EngineConfig config_from(const gr_batch_options* o, uint32_t width, const std::vector<const gr_job*>& jobs) {
    EngineConfig cfg;
    cfg.width = width;
    if (o && o->path_capacity) {
        cfg.capacity = o->path_capacity;
    } else {
        uint64_t samples = 0;
        for (const gr_job* j : jobs) samples += static_cast<uint64_t>(j->film->width) * j->film->height * j->params.spp;
        cfg.capacity = 1u << 20;
        while (cfg.capacity < samples && cfg.capacity < (1u << 26)) cfg.capacity <<= 1;
    }
    if (o && o->block_size) cfg.block = o->block_size;
    return cfg;
}

}  // namespace

extern "C" {

gr_status gr_render_batch(const gr_job* jobs, uint32_t n, const gr_batch_options* options) {
    if (n && !jobs) {
        set_error("null jobs");
        return GR_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> g(g_cache_mu);
    g_batch_stats = gr_render_stats{};
    std::map<uint32_t, std::vector<const gr_job*>> by_width;
    std::vector<const gr_job*> sequential;
    for (uint32_t i = 0; i < n; ++i) {
        gr_status s = check_job(jobs[i]);
        if (s != GR_OK) return s;
        if (jobs[i].params.integrator == GR_INTEGRATOR_BDPT) sequential.push_back(&jobs[i]);
        else by_width[jobs[i].scene->dev.width].push_back(&jobs[i]);
    }
    for (auto& kv : by_width) {
        gr_status s = run_engine_batch(kv.second, config_from(options, kv.first, kv.second), g_batch_stats, nullptr);
        if (s != GR_OK) return s;
        for (const gr_job* j : kv.second) j->film->passes += j->params.spp;
    }
    // BDPT keeps its own per-image wavefront.
    for (const gr_job* j : sequential) {
        gr_status s = gr_render(j->scene, &j->camera, &j->params, j->film);
        if (s != GR_OK) return s;
        g_batch_stats.samples += j->scene->stats.samples;
        g_batch_stats.extension_rays += j->scene->stats.extension_rays;
        g_batch_stats.shadow_rays += j->scene->stats.shadow_rays;
        g_batch_stats.device_ms += j->scene->stats.device_ms;
    }
    return GR_OK;
}

gr_status gr_batch_release(void) {
    std::lock_guard<std::mutex> g(g_cache_mu);
    g_cache.clear();  // each engine waits for its stream, then frees its buffers
    g_cache_used.clear();
    return GR_OK;
}

gr_status gr_batch_last_stats(gr_render_stats* out) {
    if (!out) {
        set_error("null argument");
        return GR_ERR_INVALID_ARGUMENT;
    }
    *out = g_batch_stats;
    return GR_OK;
}

gr_status gr_batch_autotune(const gr_job* jobs, uint32_t n, gr_batch_options* out) {
    if (!out || (n && !jobs)) {
        set_error("null argument");
        return GR_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> g(g_cache_mu);
    // Trial: the first four passes of up to 64 path-tracer jobs of the most common width,
    // rendered into scratch films.
    std::map<uint32_t, std::vector<const gr_job*>> by_width;
    for (uint32_t i = 0; i < n; ++i) {
        gr_status s = check_job(jobs[i]);
        if (s != GR_OK) return s;
        if (jobs[i].params.integrator != GR_INTEGRATOR_BDPT) by_width[jobs[i].scene->dev.width].push_back(&jobs[i]);
    }
    std::memset(out, 0, sizeof(*out));
    out->use_graph = 1;
    if (by_width.empty()) return GR_OK;
    auto best_w = std::max_element(by_width.begin(), by_width.end(),
                                   [](auto& a, auto& b) { return a.second.size() < b.second.size(); });
    std::vector<gr_job> trial;
    for (size_t k = 0; k < best_w->second.size() && k < 64; ++k) {
        gr_job j = *best_w->second[k];
        j.params.spp = std::min<uint32_t>(j.params.spp, 4);
        trial.push_back(j);
    }
    std::vector<DevBuf> films(trial.size());
    std::vector<float4*> fp(trial.size());
    for (size_t k = 0; k < trial.size(); ++k) {
        size_t bytes = static_cast<size_t>(trial[k].film->width) * trial[k].film->height * sizeof(float4);
        GR_CUDA_TRY(films[k].ensure(bytes));
        GR_CUDA_TRY(cudaMemset(films[k].ptr, 0, bytes));
        fp[k] = films[k].as<float4>();
    }
    std::vector<const gr_job*> tj;
    for (auto& j : trial) tj.push_back(&j);
    double best = 0.0;
    // Path capacity (queue size; the state ring is about twice it) and extension block
    // size.  Larger capacities amortise the per-iteration launches and the tail of the
    // last units: on the serving scenes' requests 16 M -> 32 M -> 64 M measured 1578 ->
    // 1681 -> 1764 Msamples/s.
    for (uint32_t cap : {1u << 23, 1u << 25, 1u << 26}) {
        for (uint32_t bs : {128u, 256u}) {
            EngineConfig cfg;
            cfg.width = best_w->first;
            cfg.capacity = cap;
            cfg.block = bs;
            gr_render_stats st{};
            gr_status s = run_engine_batch(tj, cfg, st, fp.data());  // warm (engine set-up)
            if (s != GR_OK) return s;
            st = gr_render_stats{};
            s = run_engine_batch(tj, cfg, st, fp.data());
            if (s != GR_OK) return s;
            double rate = st.device_ms > 0 ? st.samples / st.device_ms : 0.0;
            if (rate > best) {
                best = rate;
                out->path_capacity = cap;
                out->block_size = bs;
            }
        }
    }
    return GR_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------ serving

struct ServerRequest {
    uint64_t id;
    gr_request req;
    int32_t state;
    DevBuf film;
    uint32_t job = 0;
    uint32_t appended = 0;  // passes appended to the engine so far
    std::vector<uint32_t> units;  // engine unit indices, in pass order
    uint32_t passes_done = 0;
    double submit_ms = 0, start_ms = 0, finish_ms = 0;
    uint64_t bytes = 0;
    bool admitted = false;  // its job is in the engine
    // Progressive refinement: even passes go to `film` (job), odd passes to `film2`
    // (job2); passes are appended up to `limit`, the next checkpoint (next_checkpoint).
    bool progressive = false;
    DevBuf film2;
    uint32_t job2 = 0;
    uint32_t limit = 0;
    float rel_mse = 0.0f;
    uint32_t cap() const { return progressive ? limit : req.params.spp; }
};

constexpr uint32_t FIRST_CHECKPOINT = 8;

// The checkpoint after `done` passes of a progressive request whose error estimate `est`
// is above `target`.  The estimate falls about as 1 / passes, so the next checkpoint is
// the pass count expected to meet the target with a 10% margin, at least 1.25x and at
// most 8x `done`, rounded up to a multiple of 8 (both half-films get whole passes) and
// at most `cap` (the request's spp).  An infinite estimate takes the 8x step, a NaN one
// the 1.25x step.
uint32_t next_checkpoint(uint32_t done, float est, float target, uint32_t cap) {
    double want = static_cast<double>(done) * static_cast<double>(est) / static_cast<double>(target) * 1.1;
    const double lo = 1.25 * done, hi = 8.0 * done;
    if (!(want >= lo)) want = lo;
    if (want > hi) want = hi;
    const uint64_t n = (static_cast<uint64_t>(std::ceil(want)) + 7) / 8 * 8;
    return static_cast<uint32_t>(std::min<uint64_t>(n, cap));
}
// Aging of the shortest-remaining-work order.  On the saturated progressive serving
// workload (24 requests, relMSE 1e-3) p50 / p95 / p99 latency measured 1540 / 4210 /
// 5612 ms without aging, 1507 / 4120 / 4207 at 1000 ms and 1653 / 3693 / 4066 at 250 ms.
#ifndef GR_SERVE_AGE_MS
#define GR_SERVE_AGE_MS 1000.0
#endif
constexpr double SERVE_AGE_MS = GR_SERVE_AGE_MS;
constexpr int EST_BLOCKS = 256;

// Per-block sums of |a - b|^2 and |(accum_a + accum_b) / (weight_a + weight_b)|^2 over the
// pixels of two half-films (a, b = accum / weight); pixels without weight are skipped.
// Fixed blocks and an in-order host sum keep the estimate the same from run to run.
__global__ void __launch_bounds__(256) k_half_film_error(const float4* __restrict__ a, const float4* __restrict__ b,
                                                         uint32_t n, double2* __restrict__ partial) {
    double d = 0.0, m = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 pa = a[i], pb = b[i];
        if (!(pa.w > 0.0f) || !(pb.w > 0.0f)) continue;
        double ax = pa.x / pa.w, ay = pa.y / pa.w, az = pa.z / pa.w;
        double bx = pb.x / pb.w, by = pb.y / pb.w, bz = pb.z / pb.w;
        double w = static_cast<double>(pa.w) + pb.w;
        double fx = (static_cast<double>(pa.x) + pb.x) / w, fy = (static_cast<double>(pa.y) + pb.y) / w,
               fz = (static_cast<double>(pa.z) + pb.z) / w;
        d += (ax - bx) * (ax - bx) + (ay - by) * (ay - by) + (az - bz) * (az - bz);
        m += fx * fx + fy * fy + fz * fz;
    }
    __shared__ double sd[256], sm[256];
    sd[threadIdx.x] = d;
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (static_cast<int>(threadIdx.x) < o) {
            sd[threadIdx.x] += sd[threadIdx.x + o];
            sm[threadIdx.x] += sm[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = make_double2(sd[0], sm[0]);
}

struct gr_server {
    std::mutex mu;
    Engine engine;
    gr_server_options opts{};
    uint64_t budget = 0, used = 0;
    uint64_t next_id = 1;
    std::vector<std::unique_ptr<ServerRequest>> reqs;
    // Scenes of taken requests that were cancelled while running: their paths may still
    // be queued, so the scene is released once the engine reports all work gathered.
    std::vector<gr_scene*> retired;
    uint64_t resets = 0;  // times the engine's job and unit tables were cleared at idle
    double pair_ms = 0.0;  // moving average of one graph pair's wall time, for step sizing
    std::chrono::steady_clock::time_point t0;
    double now_ms() const {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    ServerRequest* find(uint64_t id) {
        for (auto& r : reqs)
            if (r->id == id) return r.get();
        return nullptr;
    }
};

namespace {

// Admits queued requests while films fit the budget, then tops up the engine's unit
// backlog (continuous batching: a request that arrives is admitted and appended at the
// next step, while the earlier ones are still on the GPU).
gr_status schedule(gr_server* s) {
    uint32_t active = 0;
    for (auto& r : s->reqs) active += r->state == GR_REQUEST_RUNNING ? 1 : 0;
    for (auto& r : s->reqs) {
        if (r->state != GR_REQUEST_QUEUED) continue;
        if (s->opts.max_active && active >= s->opts.max_active) break;
        if (s->used + r->bytes > s->budget) break;  // admission by free device memory, in arrival order
        gr_status st;
        const size_t film_bytes = r->progressive ? r->bytes / 2 : r->bytes;
        GR_CUDA_TRY(r->film.ensure(film_bytes));
        GR_CUDA_TRY(cudaMemset(r->film.ptr, 0, film_bytes));
        DevJob dj = make_job(r->req.scene, r->req.camera, r->req.params, r->req.width, r->req.height,
                             r->film.as<float4>());
        st = s->engine.add_job(dj, 0, 0, r->job);
        if (st != GR_OK) return st;
        if (r->progressive) {
            const size_t half = r->bytes / 2;
            GR_CUDA_TRY(r->film2.ensure(half));
            GR_CUDA_TRY(cudaMemset(r->film2.ptr, 0, half));
            DevJob d2 = make_job(r->req.scene, r->req.camera, r->req.params, r->req.width, r->req.height,
                                 r->film2.as<float4>());
            st = s->engine.add_job(d2, 0, 0, r->job2);
            if (st != GR_OK) return st;
        }
        s->used += r->bytes;
        r->state = GR_REQUEST_RUNNING;
        r->admitted = true;
        r->start_ms = s->now_ms();
        ++active;
    }
    // Keep about two pools' worth of paths appended but not yet issued (from the control
    // block the last run read: only this function appends, and it runs before each run).
    const EngineCtl& c = s->engine.last_ctl();
    gr_status st = GR_OK;
    uint64_t backlog = c.paths_total - c.gcur;
    const uint64_t want = 2ull * s->engine.capacity();
    // Which request's passes go first (gr_server_options.policy):
    //   arrival order: the oldest request's; a later request's passes are appended only
    //     when the older ones have nothing left to append within the backlog, so they
    //     fill the paths the older ones leave free (a FIFO with backfill);
    //   shortest first: the request with the fewest samples left, divided by
    //     1 + (time since submission) / SERVE_AGE_MS, so a long request's priority grows
    //     as it waits.
    const double now = s->now_ms();
    const bool shortest = s->opts.policy == GR_SERVE_SHORTEST_FIRST;
    std::vector<std::pair<double, ServerRequest*>> order;
    for (auto& r : s->reqs)
        if (r->state == GR_REQUEST_RUNNING && r->appended < r->cap()) {
            const double left = static_cast<double>(r->cap() - r->appended) * r->req.width * r->req.height;
            order.emplace_back(shortest ? left / (1.0 + (now - r->submit_ms) / SERVE_AGE_MS) : r->submit_ms,
                               r.get());
        }
    std::stable_sort(order.begin(), order.end(),
                     [](const std::pair<double, ServerRequest*>& a, const std::pair<double, ServerRequest*>& b) {
                         return a.first < b.first;
                     });
    std::vector<std::pair<uint32_t, uint32_t>> batch;
    std::vector<ServerRequest*> owners;
    for (auto& o : order) {
        ServerRequest* r = o.second;
        while (backlog < want && r->appended < r->cap()) {
            const bool odd = r->progressive && (r->appended & 1u);
            batch.emplace_back(odd ? r->job2 : r->job, r->req.params.first_pass + r->appended);
            owners.push_back(r);
            r->appended += 1;
            backlog += static_cast<uint64_t>(r->req.width) * r->req.height;
        }
        if (backlog >= want) break;
    }
    if (!batch.empty()) {
        size_t first = s->engine.units().size();
        st = s->engine.append_units(batch);
        if (st != GR_OK) return st;
        for (size_t k = 0; k < owners.size(); ++k) owners[k]->units.push_back(static_cast<uint32_t>(first + k));
    }
    return GR_OK;
}

// relMSE estimate of a progressive request's image from its two half-films: the
// half-images a and b are independent estimates with variance v each, so E|a - b|^2 = 2v
// and the full image (variance v / 2) has MSE ~ sum |a - b|^2 / 4.
gr_status half_film_rel_mse(gr_server* s, const ServerRequest& r, float& out) {
    DevBuf partial;
    GR_CUDA_TRY(partial.ensure(EST_BLOCKS * sizeof(double2)));
    const uint32_t n = r.req.width * r.req.height;
    cudaStream_t st = s->engine.stream();
    k_half_film_error<<<EST_BLOCKS, 256, 0, st>>>(r.film.as<float4>(), r.film2.as<float4>(), n,
                                                 partial.as<double2>());
    GR_CUDA_TRY(cudaGetLastError());
    std::vector<double2> h(EST_BLOCKS);
    GR_CUDA_TRY(cudaMemcpyAsync(h.data(), partial.ptr, EST_BLOCKS * sizeof(double2), cudaMemcpyDeviceToHost, st));
    GR_CUDA_TRY(cudaStreamSynchronize(st));
    double d = 0.0, m = 0.0;
    for (const double2& v : h) {
        d += v.x;
        m += v.y;
    }
    out = m > 0.0 ? static_cast<float>(d / 4.0 / m) : 0.0f;
    return GR_OK;
}

// With no request running and every appended unit gathered, no path of any job is left
// on the device: the scenes of retired requests are released and the engine's job and
// unit tables are cleared, so a long-running server does not grow them with everything
// it has served.  Finished requests keep their films (their own buffers) until taken.
gr_status reset_if_idle(gr_server* s) {
    if (s->engine.units().empty() && s->engine.jobs().empty()) return GR_OK;
    for (auto& r : s->reqs)
        if (r->state == GR_REQUEST_RUNNING) return GR_OK;
    EngineCtl c;
    gr_status st = s->engine.read_ctl(c);
    if (st != GR_OK) return st;
    if (c.g_lo != c.units_count) return GR_OK;
    for (gr_scene* sc : s->retired) scene_release(sc);
    s->retired.clear();
    st = s->engine.reset();
    if (st != GR_OK) return st;
    for (auto& r : s->reqs) r->units.clear();  // indices into the cleared table
    s->resets += 1;
    return GR_OK;
}

// Marks passes gathered (every unit below the engine's g_lo is in its film).
gr_status progress(gr_server* s) {
    const EngineCtl& c = s->engine.last_ctl();  // as the last run left it
    gr_status st = GR_OK;
    for (auto& r : s->reqs) {
        if (r->state != GR_REQUEST_RUNNING) continue;
        uint32_t d = 0;
        for (uint32_t u : r->units) d += u < c.g_lo ? 1 : 0;
        r->passes_done = d;
        if (d != r->cap()) continue;
        if (r->progressive) {  // a checkpoint: estimate the error from the two half-films
            st = half_film_rel_mse(s, *r, r->rel_mse);
            if (st != GR_OK) return st;
            if (!(r->rel_mse <= r->req.target_rel_mse) && r->limit < r->req.params.spp) {
                r->limit = next_checkpoint(r->limit, r->rel_mse, r->req.target_rel_mse, r->req.params.spp);
                continue;
            }
        }
        r->state = GR_REQUEST_DONE;
        r->finish_ms = s->now_ms();
    }
    return GR_OK;
}

}  // namespace

extern "C" {

gr_status gr_server_create(const gr_server_options* o, gr_server** out) {
    if (!out) {
        set_error("null argument");
        return GR_ERR_INVALID_ARGUMENT;
    }
    std::unique_ptr<gr_server> s(new gr_server());
    if (o) s->opts = *o;
    if (s->opts.policy != GR_SERVE_ARRIVAL_ORDER && s->opts.policy != GR_SERVE_SHORTEST_FIRST) {
        set_error("unknown serving policy");
        return GR_ERR_INVALID_ARGUMENT;
    }
    EngineConfig cfg;
    // 64 M paths in flight (about 18 GB of queues and path ring): on the serving
    // scenes' requests 16 M -> 32 M -> 64 M measured 1505 -> 1654 -> 1728 Msamples/s.
    cfg.capacity = s->opts.path_capacity ? s->opts.path_capacity : (1u << 26);
    cfg.width = s->opts.bvh_width ? s->opts.bvh_width : 4;
    cfg.block = s->opts.block_size ? s->opts.block_size : 128;
    gr_status st = s->engine.init(cfg, nullptr);
    if (st != GR_OK) return st;
    size_t free_b = 0, total_b = 0;
    GR_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    s->budget = s->opts.memory_budget_bytes ? s->opts.memory_budget_bytes : static_cast<uint64_t>(0.9 * free_b);
    s->t0 = std::chrono::steady_clock::now();
    *out = s.release();
    return GR_OK;
}

gr_status gr_server_destroy(gr_server* s) {
    if (!s) return GR_OK;
    std::vector<gr_scene*> held;
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->engine.stream()) cudaStreamSynchronize(s->engine.stream());
        held = s->retired;
        for (auto& r : s->reqs) held.push_back(r->req.scene);
    }
    delete s;  // the engine's buffers go first; then no path can reach the scenes
    for (gr_scene* sc : held) scene_release(sc);
    return GR_OK;
}

gr_status gr_server_submit(gr_server* s, const gr_request* r, uint64_t* id) {
    if (!s || !r || !id || !r->scene || r->width == 0 || r->height == 0) {
        set_error("bad request");
        return GR_ERR_INVALID_ARGUMENT;
    }
    if (r->params.integrator == GR_INTEGRATOR_BDPT) {
        set_error("the serving loop runs the path tracer and the display-colour integrator");
        return GR_ERR_UNSUPPORTED;
    }
    if (r->scene->dev.width != s->engine.config().width) {
        set_error("request scene has a different BVH width than the server");
        return GR_ERR_INVALID_ARGUMENT;
    }
    if (static_cast<uint64_t>(r->width) * r->height * 2 > s->engine.ring()) {
        set_error("request image too large for the server's path ring (raise path_capacity)");
        return GR_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> g(s->mu);
    std::unique_ptr<ServerRequest> q(new ServerRequest());
    q->id = s->next_id++;
    q->req = *r;
    q->state = r->params.spp ? GR_REQUEST_QUEUED : GR_REQUEST_DONE;
    q->bytes = static_cast<uint64_t>(r->width) * r->height * sizeof(float4);
    if (!(r->target_rel_mse >= 0.0f)) {
        set_error("target_rel_mse must be >= 0");
        return GR_ERR_INVALID_ARGUMENT;
    }
    if (r->target_rel_mse > 0.0f) {  // two half-films
        q->progressive = true;
        q->bytes *= 2;
        q->limit = std::min(FIRST_CHECKPOINT, r->params.spp);
    }
    q->submit_ms = s->now_ms();
    if (q->bytes > s->budget) {
        set_error("request film exceeds the server's memory budget");
        return GR_ERR_OUT_OF_MEMORY;
    }
    *id = q->id;
    scene_retain(r->scene);  // until the request is taken (or the server destroyed)
    s->reqs.push_back(std::move(q));
    return GR_OK;
}

gr_status gr_server_step(gr_server* s, double budget_ms) {
    if (!s) {
        set_error("null server");
        return GR_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> g(s->mu);
    double t_end = s->now_ms() + budget_ms;
    for (;;) {
        gr_status st = schedule(s);
        if (st != GR_OK) return st;
        bool any = false;
        for (auto& r : s->reqs) any |= r->state == GR_REQUEST_RUNNING;
        if (!any) return reset_if_idle(s);
        // As many pairs as the step's budget allows (from the time pairs have taken so
        // far; at least 1, at most 4), ending early once every unit of the running
        // request that completes first in unit order is gathered, so the host hears of
        // finished requests (and takes new ones) within about one pair.
        uint32_t stop = 0xFFFFFFFFu;
        for (auto& r : s->reqs)
            if (r->state == GR_REQUEST_RUNNING && r->appended == r->cap() && !r->units.empty())
                stop = std::min(stop, r->units.back() + 1);
        const double left = t_end - s->now_ms();
        uint32_t pairs = 4;
        if (s->pair_ms > 0.0) pairs = static_cast<uint32_t>(std::max(1.0, std::min(4.0, left / s->pair_ms)));
        st = s->engine.set_flush_unit(stop == 0xFFFFFFFFu ? 0u : stop);
        if (st != GR_OK) return st;
        bool done = false;
        const double t_run = s->now_ms();
        st = s->engine.run(pairs, done, stop);
        if (st != GR_OK) return st;
        if (s->engine.last_pairs() > 0) {
            const double per = (s->now_ms() - t_run) / s->engine.last_pairs();
            s->pair_ms = s->pair_ms > 0.0 ? 0.7 * s->pair_ms + 0.3 * per : per;
        }
        if (done && !s->retired.empty()) {  // every appended unit gathered: no path left
            GR_CUDA_TRY(cudaStreamSynchronize(s->engine.stream()));
            for (gr_scene* sc : s->retired) scene_release(sc);
            s->retired.clear();
        }
        st = progress(s);
        if (st != GR_OK) return st;
        if (s->now_ms() >= t_end) return GR_OK;
    }
}

gr_status gr_server_poll(gr_server* s, uint64_t id, gr_request_status* out) {
    if (!s || !out) {
        set_error("null argument");
        return GR_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> g(s->mu);
    ServerRequest* r = s->find(id);
    if (!r) {
        set_error("no such request");
        return GR_ERR_NOT_FOUND;
    }
    out->state = r->state;
    out->passes_done = r->passes_done;
    out->submit_ms = r->submit_ms;
    out->start_ms = r->start_ms;
    out->finish_ms = r->finish_ms;
    out->rel_mse = r->rel_mse;
    out->reserved = 0;
    return GR_OK;
}

gr_status gr_server_cancel(gr_server* s, uint64_t id) {
    if (!s) {
        set_error("null server");
        return GR_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> g(s->mu);
    ServerRequest* r = s->find(id);
    if (!r) {
        set_error("no such request");
        return GR_ERR_NOT_FOUND;
    }
    if (r->state == GR_REQUEST_RUNNING) {
        gr_status st = s->engine.cancel_job(r->job);
        if (st != GR_OK) return st;
        if (r->progressive) {
            st = s->engine.cancel_job(r->job2);
            if (st != GR_OK) return st;
            r->limit = r->appended;
        }
        // Its appended units still drain (paths die on their next shade; the gather
        // skips the film); no further passes are appended.
        r->req.params.spp = r->appended;
    }
    if (r->state == GR_REQUEST_QUEUED || r->state == GR_REQUEST_RUNNING) {
        r->state = GR_REQUEST_CANCELLED;
        r->finish_ms = s->now_ms();
    }
    return GR_OK;
}

// Copies a request's film to host arrays (accum: 3 floats per pixel, weight: 1; either
// may be null), a progressive request's two half-films summed; zeros before admission.
static gr_status copy_film(gr_server* s, const ServerRequest& r, float* accum, float* weight) {
    if (!accum && !weight) return GR_OK;
    const size_t n = static_cast<size_t>(r.req.width) * r.req.height;
    std::vector<float4> px(n, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    if (r.film.ptr) {
        GR_CUDA_TRY(cudaStreamSynchronize(s->engine.stream()));
        GR_CUDA_TRY(cudaMemcpy(px.data(), r.film.ptr, n * sizeof(float4), cudaMemcpyDeviceToHost));
        if (r.progressive && r.film2.ptr) {  // even + odd passes
            std::vector<float4> p2(n);
            GR_CUDA_TRY(cudaMemcpy(p2.data(), r.film2.ptr, n * sizeof(float4), cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < n; ++i)
                px[i] = make_float4(px[i].x + p2[i].x, px[i].y + p2[i].y, px[i].z + p2[i].z, px[i].w + p2[i].w);
        }
    }
    for (size_t i = 0; i < n; ++i) {
        if (accum) {
            accum[3 * i] = px[i].x;
            accum[3 * i + 1] = px[i].y;
            accum[3 * i + 2] = px[i].z;
        }
        if (weight) weight[i] = px[i].w;
    }
    return GR_OK;
}

gr_status gr_server_snapshot(gr_server* s, uint64_t id, float* accum, float* weight, uint32_t* passes) {
    if (!s) {
        set_error("null server");
        return GR_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> g(s->mu);
    ServerRequest* r = s->find(id);
    if (!r) {
        set_error("no such request");
        return GR_ERR_NOT_FOUND;
    }
    if (passes) *passes = r->passes_done;
    return copy_film(s, *r, accum, weight);
}

gr_status gr_server_get_info(gr_server* s, gr_server_info* out) {
    if (!s || !out) {
        set_error("null argument");
        return GR_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> g(s->mu);
    std::memset(out, 0, sizeof(*out));
    for (auto& r : s->reqs) {
        if (r->state == GR_REQUEST_QUEUED) out->queued += 1;
        else if (r->state == GR_REQUEST_RUNNING) out->running += 1;
        else out->finished += 1;
    }
    out->engine_jobs = static_cast<uint32_t>(s->engine.jobs().size());
    out->engine_units = s->engine.units().size();
    out->resets = s->resets;
    out->film_bytes = s->used;
    out->memory_budget_bytes = s->budget;
    return GR_OK;
}

gr_status gr_server_take(gr_server* s, uint64_t id, float* accum, float* weight) {
    if (!s) {
        set_error("null server");
        return GR_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> g(s->mu);
    for (size_t k = 0; k < s->reqs.size(); ++k) {
        ServerRequest* r = s->reqs[k].get();
        if (r->id != id) continue;
        if (r->state != GR_REQUEST_DONE && r->state != GR_REQUEST_CANCELLED) {
            set_error("request not finished");
            return GR_ERR_BUSY;
        }
        gr_status cst = copy_film(s, *r, accum, weight);
        if (cst != GR_OK) return cst;
        // A finished request's units are all gathered, and one never admitted has no
        // paths: its scene can go.  One cancelled while running may still have paths
        // draining.  (Nothing is changed before the last call that can fail.)
        const bool drained = r->state == GR_REQUEST_DONE || !r->admitted;
        if (drained) GR_CUDA_TRY(cudaStreamSynchronize(s->engine.stream()));
        if (r->film.ptr) s->used -= r->bytes;
        if (drained)
            scene_release(r->req.scene);
        else
            s->retired.push_back(r->req.scene);
        s->reqs.erase(s->reqs.begin() + static_cast<long>(k));
        return GR_OK;
    }
    set_error("no such request");
    return GR_ERR_NOT_FOUND;
}

}  // extern "C"
