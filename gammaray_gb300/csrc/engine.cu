// Multi-job wavefront engine (see engine.hpp): kernels, graph capture and host driver.
#include <algorithm>
#include <cstring>

#include "engine.hpp"
#include "film_gather.cuh"
#include "shade_sort.cuh"
#include "traverse.cuh"

namespace gr {

namespace {

constexpr int EBLOCK = 128;
// The engine's shading kernel: blocks of GR_ENG_SHADE_BLOCK threads (128 or 768), each
// sorting its chunk of the queue by code path.  At 768 one block fills an SM (85
// registers), so all of an SM's warps shade the same code path at a time, as in the
// path tracer's k_shade.
#ifndef GR_ENG_SHADE_BLOCK
#define GR_ENG_SHADE_BLOCK 768
#endif
constexpr int ESBLOCK = GR_ENG_SHADE_BLOCK;
static_assert(ESBLOCK == 128 || ESBLOCK == 768, "engine shading block of 128 or 768 threads");
constexpr uint32_t ESHADE_PER_THREAD = ESBLOCK == 128 ? SHADE_PER_THREAD : SHADE_BIG_PER;

// Path state.  The queue entry of a live path carries its ray, its job (o.w), its depth
// (d.w) and its state, two float4:
//   state[2q]     = (throughput.xyz, radiance.x)
//   state[2q + 1] = (radiance.y, radiance.z, key low 32 bits, key high 32 bits)
// read where the entry is shaded and written where the surviving path is pushed.  Global
// path p (the paths of all units, in unit order) has ring slot p & (ring - 1):
//   s_hot[slot]  = (radiance.xyz, 0), written when the path finishes
//   s_cold[slot] = (unit, 0, film s bits, film t bits), written when it starts
// The gather reads a finished unit's samples straight from its slots, so a slot is
// reused only once the unit of its previous path is gathered: paths are issued up to
// `ring` past the oldest ungathered one.  At most `capacity` paths are live (the queues'
// size).
GR_D uint64_t state_key(float4 b) {
    return (static_cast<uint64_t>(__float_as_uint(b.w)) << 32) | __float_as_uint(b.z);
}

GR_D void push_ray(bool alive, uint32_t* count_out, uint32_t slot, V3 o, V3 d, uint32_t job, uint32_t depth,
                   float4 sa, float4 sb, uint32_t* __restrict__ nslot, float4* __restrict__ no,
                   float4* __restrict__ nd, float4* __restrict__ nstate, uint32_t cap) {
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
        no[pos] = make_float4(o.x, o.y, o.z, __uint_as_float(job));
        nd[pos] = make_float4(d.x, d.y, d.z, __uint_as_float(depth));
        nstate[2 * static_cast<size_t>(pos)] = sa;
        nstate[2 * static_cast<size_t>(pos) + 1] = sb;
    }
}

// The unit holding global path p: the last unit whose prefix is <= p.
GR_D uint32_t find_unit(const DevUnit* __restrict__ units, uint32_t lo, uint32_t hi, unsigned long long p) {
    while (hi - lo > 1) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (units[mid].prefix <= p) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Single thread: what to gather and how many paths to issue this iteration.
__global__ void k_eng_plan(EngineCtl* c, const DevJob* __restrict__ jobs, const DevUnit* __restrict__ units,
                           const uint32_t* __restrict__ unit_done, uint32_t cap, uint32_t ring, int cur) {
    // Finished units, consecutive from the oldest, grouped by job (pass order kept).
    uint32_t u = c->g_lo, n = 0, groups = 0;
    uint32_t gjob[GATHER_MAX];
    uint32_t tmp[GATHER_MAX];
    uint32_t tmp_group[GATHER_MAX];
    while (u < c->units_count && n < GATHER_MAX) {
        DevUnit U = units[u];
        if (unit_done[u] < U.npix) break;
        uint32_t g = 0;
        while (g < groups && gjob[g] != U.job) ++g;
        if (g == groups) {
            gjob[groups] = U.job;
            c->gather_group_count[groups] = 0;
            ++groups;
        }
        c->gather_group_count[g] += 1;
        tmp[n] = u;
        tmp_group[n] = g;
        ++n;
        ++u;
    }
    // Gather in larger batches: a call adds several passes per film tile, so the
    // film's read-modify-write and the staging prologue are paid once for them.  Wait
    // until half a capacity of finished paths is waiting, unless the unit list is full,
    // every appended unit has finished, or the ring would soon limit the fill.
    const unsigned long long fin = (u < c->units_count ? units[u].prefix : c->paths_total) - c->gather_lo_prefix;
    const bool flush = n == GATHER_MAX || u == c->units_count || fin >= cap / 2 ||
                       c->gcur + cap > c->gather_lo_prefix + ring || (c->flush_unit != 0 && u >= c->flush_unit);
    if (!flush) {
        n = 0;
        groups = 0;
        u = c->g_lo;
    }
    uint32_t first = 0, tiles = 0;
    for (uint32_t g = 0; g < groups; ++g) {
        c->gather_group_first[g] = first;
        c->gather_group_tiles[g] = tiles;
        const DevJob& J = jobs[gjob[g]];
        tiles += film_tiles_x(J.width) * film_tiles_y(J.height);
        first += c->gather_group_count[g];
    }
    uint32_t fill[GATHER_MAX];
    for (uint32_t g = 0; g < groups; ++g) fill[g] = c->gather_group_first[g];
    for (uint32_t k = 0; k < n; ++k) c->gather_units[fill[tmp_group[k]]++] = tmp[k];
    c->gather_n = n;
    c->gather_groups = groups;
    c->gather_tiles = tiles;
    c->g_lo = u;
    c->gather_lo_prefix = u < c->units_count ? units[u].prefix : c->paths_total;
    // Every live path has its next ray in the current queue (the last shade's survivors).
    unsigned long long live = c->q[cur];
    unsigned long long room = cap > live ? cap - live : 0;
    unsigned long long rem = c->paths_total - c->gcur;
    unsigned long long lim = c->gather_lo_prefix + ring - c->gcur;  // ring slots free of ungathered samples
    unsigned long long nf = min(room, min(rem, lim));
    c->fill_n = static_cast<uint32_t>(nf);
    c->fill_base = c->gcur;
    // The fill's camera rays go after the last shade's survivors, at fixed positions.
    c->fill_qbase = c->q[cur];
    c->q[cur] += static_cast<uint32_t>(nf);
    if (nf) {  // every unit before g_lo is issued, so the fill starts at or after it
        c->fill_ulo = find_unit(units, c->g_lo, c->units_count, c->gcur);
        c->fill_uhi = find_unit(units, c->fill_ulo, c->units_count, c->gcur + nf - 1);
    }
    c->gcur += nf;
    c->done = c->g_lo == c->units_count ? 1u : 0u;
    c->iter += 1;
    c->fetch = 0;  // the extension kernel of this iteration starts handing out rays at 0
    c->gather_next = 0;  // and the gather its film-tile items
}

// A unit's samples in their ring slots.
struct RingSamples {
    const float4* __restrict__ hot;
    const uint4* __restrict__ cold;
    unsigned long long prefix;
    uint32_t width, mask;
    GR_D void operator()(uint32_t r, uint32_t col, float2& st, V3& rgb) const {
        size_t slot = static_cast<size_t>((prefix + static_cast<unsigned long long>(r) * width + col) & mask);
        float4 a = hot[slot];  // (radiance, 0) of the finished path
        uint4 cd = cold[slot];
        st = make_float2(__uint_as_float(cd.z), __uint_as_float(cd.w));
        rgb = V3{a.x, a.y, a.z};
    }
};

__global__ void __launch_bounds__(FILM_THREADS, GR_FILM_BLOCKS_PER_SM)
    k_eng_gather(EngineCtl* c, const DevJob* __restrict__ jobs, const DevUnit* __restrict__ units,
                 const float4* __restrict__ s_hot, const uint4* __restrict__ s_cold, uint32_t mask) {
    __shared__ StagedSample sm;
    __shared__ uint32_t s_item;
    const uint32_t total = c->gather_tiles, groups = c->gather_groups;
    // Items (a job's film tile and its finished passes) are taken from a counter: their
    // pass counts differ, so a fixed stride would leave blocks idle.
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(&c->gather_next, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        __syncthreads();  // every thread has read s_item before it is taken again
        if (item >= total) break;
        uint32_t g = 0;
        while (g + 1 < groups && c->gather_group_tiles[g + 1] <= item) ++g;
        const uint32_t t = item - c->gather_group_tiles[g];
        const uint32_t first = c->gather_group_first[g], cnt = c->gather_group_count[g];
        const DevJob& J = jobs[units[c->gather_units[first]].job];
        const uint32_t w = J.width, h = J.height;
        const uint32_t tx = film_tiles_x(w);
        const int ox = static_cast<int>((t % tx) * FILM_TILE_W), oy = static_cast<int>((t / tx) * FILM_TILE_H);
        const int x = ox + threadIdx.x % FILM_TILE_W, y = oy + threadIdx.x / FILM_TILE_W;
        const bool inside = x < static_cast<int>(w) && y < static_cast<int>(h);
        float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (inside) acc = J.film[static_cast<size_t>(y) * w + x];
        gather_passes(sm, w, h, ox, oy, acc, cnt, [&](uint32_t k) {  // the job's passes, in order
            return RingSamples{s_hot, s_cold, units[c->gather_units[first + k]].prefix, w, mask};
        });
        if (inside && J.live) J.film[static_cast<size_t>(y) * w + x] = acc;
    }
}

// Starts the next fill_n paths in their ring slots (coalesced: consecutive paths,
// consecutive slots) and queues their camera rays at the positions the plan reserved
// (no atomics).
__global__ void __launch_bounds__(EBLOCK) k_eng_fill(EngineCtl* c, const DevJob* __restrict__ jobs,
                                                     const DevUnit* __restrict__ units, uint32_t mask,
                                                     uint4* __restrict__ s_cold, uint32_t* __restrict__ q_slot,
                                                     float4* __restrict__ q_o, float4* __restrict__ q_d,
                                                     float4* __restrict__ q_state, uint32_t cap) {
    const uint32_t n = c->fill_n, qbase = c->fill_qbase;
    const unsigned long long base = c->fill_base;
    const uint32_t ulo = c->fill_ulo, uhi = c->fill_uhi + 1;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned long long p = base + i;
        const uint32_t slot = static_cast<uint32_t>(p & mask);
        const uint32_t u = find_unit(units, ulo, uhi, p);
        const DevUnit U = units[u];
        const uint32_t pixel = static_cast<uint32_t>(p - U.prefix);
        const DevJob& J = jobs[U.job];
        const uint32_t row = pixel / J.width, col = pixel - row * J.width;
        const uint64_t key = path_key(J.seed, U.pass, pixel);
        float s, t;
        film_sample_point(J.width, J.height, row, col, key, s, t);
        V3 o, d;
        camera_ray(J.cam, s, t, o, d);
        s_cold[slot] = make_uint4(u, 0, __float_as_uint(s), __float_as_uint(t));
        if (!GR_IN_RANGE(qbase + i, cap)) continue;
        const size_t qi = qbase + i;
        q_slot[qi] = slot;
        q_o[qi] = make_float4(o.x, o.y, o.z, __uint_as_float(U.job));
        q_d[qi] = make_float4(d.x, d.y, d.z, __uint_as_float(0u));
        q_state[2 * qi] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        q_state[2 * qi + 1] = make_float4(0.0f, 0.0f, __uint_as_float(static_cast<uint32_t>(key)),
                                          __uint_as_float(static_cast<uint32_t>(key >> 32)));
    }
}

template <int W, int BS>
__global__ void __launch_bounds__(BS) k_eng_extend(EngineCtl* c, int cur, const DevJob* __restrict__ jobs,
                                                   const float4* __restrict__ q_o, const float4* __restrict__ q_d,
                                                   float4* __restrict__ q_hit) {
    extern __shared__ unsigned char smem[];
    int2 spill[MAX_STACK - SMEM_STACK];
    const StackView stk = thread_stack(smem, spill);
    const uint32_t n = c->q[cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&c->rays, static_cast<unsigned long long>(n));
    auto trace = [&](uint32_t q) {
        float4 o4 = q_o[q], d4 = q_d[q];
        const DeviceScene& s = jobs[__float_as_uint(o4.w)].scene;
        TraceResult r = trace_ray<W, false>(s, V3{o4.x, o4.y, o4.z}, V3{d4.x, d4.y, d4.z}, FLT_MAX, stk, &c->err);
        q_hit[q] = make_float4(r.t, __int_as_float(r.k), r.u, r.v);
    };
    // One ray per thread, grid-stride: grouping the engine's queue by direction (as
    // k_extend does) measured slower here (1264 -> 1207 Msamples/s on the batch).
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) trace(q);
}

// Refilling form of the engine's extension (GR_EXTEND_REFILL = k > 0), as k_extend_refill
// in wavefront.cuh: a warp hands its idle lanes new rays from c->fetch (zeroed by the
// plan) once at least k are idle; each lane keeps its ray's scene.  Every warp intrinsic
// runs at warp-uniform control flow, and the loop ends on a ballot once no ray is left.
template <int W, int BS>
__global__ void __launch_bounds__(BS) k_eng_extend_refill(EngineCtl* c, int cur, const DevJob* __restrict__ jobs,
                                                          const float4* __restrict__ q_o,
                                                          const float4* __restrict__ q_d, float4* __restrict__ q_hit) {
    extern __shared__ unsigned char smem[];
    int2 spill[MAX_STACK - SMEM_STACK];
    const StackView stk = thread_stack(smem, spill);
    const uint32_t n = c->q[cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&c->rays, static_cast<unsigned long long>(n));
    const unsigned lane = threadIdx.x & 31u;
    const unsigned below = (1u << lane) - 1u;
    TravState t;
    TraceScene s{nullptr, nullptr};
    uint32_t q = 0, steps = 0, budget = 0;
    bool busy = false, exhausted = false;
    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, !busy);
        if (!exhausted && __popc(idle) >= (GR_EXTEND_REFILL > 32 ? 32 : GR_EXTEND_REFILL)) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&c->fetch, static_cast<uint32_t>(__popc(idle)));
            base = __shfl_sync(0xffffffffu, base, 0);
            exhausted = static_cast<uint64_t>(base) + __popc(idle) >= n;
            if (!busy) {
                const uint32_t mine = base + __popc(idle & below);
                if (mine < n) {
                    float4 o4 = q_o[mine], d4 = q_d[mine];
                    const DeviceScene& js = jobs[__float_as_uint(o4.w)].scene;
                    s = TraceScene{js.nodes, js.prims};
                    budget = js.step_budget;
                    trav_init(t, V3{o4.x, o4.y, o4.z}, V3{d4.x, d4.y, d4.z}, FLT_MAX);
                    q = mine;
                    steps = 0;
                    busy = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, busy) == 0u) break;
        if (busy) {
            bool done = trav_step<W, false, false>(s, t, stk, &c->err, nullptr);
            if (!done && ++steps > budget) {
                atomicExch(&c->err, 2);
                t.hit = -1;
                done = true;
            }
            if (done) {
                q_hit[q] = make_float4(t.closest, __int_as_float(t.hit), t.hu, t.hv);
                busy = false;
            }
        }
    }
}

__global__ void __launch_bounds__(ESBLOCK, 768 / ESBLOCK)
    k_eng_shade(EngineCtl* c, int cur, const DevJob* __restrict__ jobs, uint32_t* unit_done,
                const uint32_t* __restrict__ q_slot, const float4* __restrict__ q_o,
                const float4* __restrict__ q_d, const float4* __restrict__ q_hit,
                const float4* __restrict__ q_state, float4* __restrict__ s_hot, const uint4* __restrict__ s_cold,
                uint32_t* __restrict__ nslot, float4* __restrict__ no, float4* __restrict__ nd,
                float4* __restrict__ nstate, uint32_t cap) {
    extern __shared__ unsigned char dsmem[];
    const SortView sm = sort_view<ESBLOCK, ESHADE_PER_THREAD>(dsmem);
    const int nxt = cur ^ 1;
    const uint32_t n = c->q[cur];
    const unsigned lane = threadIdx.x & 31u;
    // Material-sorted shading (shade_sort.cuh), by code path (chosen lobe type and the
    // material's lobe types, whatever the job); misses, cancelled and display-colour
    // jobs share bucket 0.  Block-uniform chunk loop.
    const uint32_t per = chunk_per_thread<ESBLOCK, ESHADE_PER_THREAD>(n, gridDim.x);
    const uint32_t chunk = chunk_entries<ESBLOCK>(n, gridDim.x, per);
    for (uint32_t c0 = blockIdx.x * chunk; c0 < n; c0 += gridDim.x * chunk) {
        const uint32_t cn = min(chunk, n - c0);
        sort_chunk<ESBLOCK, ESHADE_PER_THREAD>(sm, cn, per, [&](uint32_t i) {
            uint32_t q = c0 + i;
            uint32_t jb = __float_as_uint(q_o[q].w);
            const DevJob& J = jobs[jb];
            int32_t k = __float_as_int(q_hit[q].y);
            if (!J.live || J.display || k < 0) return 0u;
            uint64_t key = state_key(q_state[2 * static_cast<size_t>(q) + 1]);
            return shade_bucket(J.scene, k, uniform01(key, DIM_CAMERA_WALK + 4 * __float_as_uint(q_d[q].w)), 0);
        });
        for (uint32_t e = 0; e < per; ++e) {
            uint32_t i = e * ESBLOCK + threadIdx.x;
            bool alive = false, finished = false;
            uint32_t slot = 0, job = 0, unit = 0xFFFFFFFFu, depth = 0;
            V3 new_o = v3zero(), new_d = v3zero();
            float4 sa = make_float4(0.0f, 0.0f, 0.0f, 0.0f), sb = sa;
            if (i < cn) {
                uint32_t q = c0 + sm.order[i];
                slot = q_slot[q];
                float4 h = q_hit[q];
                float4 o4 = q_o[q], d4 = q_d[q];
                job = __float_as_uint(o4.w);
                depth = __float_as_uint(d4.w);
                const DevJob& J = jobs[job];
                const DeviceScene& s = J.scene;
                V3 o = V3{o4.x, o4.y, o4.z}, d = V3{d4.x, d4.y, d4.z};
                float4 ha = q_state[2 * static_cast<size_t>(q)], hb = q_state[2 * static_cast<size_t>(q) + 1];
                V3 tp = V3{ha.x, ha.y, ha.z}, L = V3{ha.w, hb.x, hb.y};
                int32_t k = __float_as_int(h.y);
                if (!J.live) {
                    // cancelled: drop the path
                } else if (k < 0) {
                    // DisplayColorIntegrator returns black on a miss (render/integrators.rs:29-31).
                    if (s.has_env && !J.display) L = L + mul(tp, V3{s.env[0], s.env[1], s.env[2]});
                } else if (J.display) {
                    uint32_t prim = __float_as_uint(__ldg(s.prims + 3 * static_cast<size_t>(k)).w);
                    const DevMaterial& m = s.materials[__ldg(s.prim_material + prim)];
                    L = V3{m.display[0], m.display[1], m.display[2]};
                } else {
                    // PathTracerIntegrator::integrate (render/integrators.rs:42-100), one segment.
                    uint32_t prim;
                    Frame f = hit_frame(s, k, o, d, h.x, h.z, h.w, prim);
                    const DevMaterial& m = s.materials[__ldg(s.prim_material + prim)];
                    uint64_t key = state_key(hb);
                    uint32_t base = DIM_CAMERA_WALK + 4 * depth;
                    MaterialSample ms = sample_world(m, -d, f, true, uniform01(key, base), uniform01(key, base + 1),
                                                     uniform01(key, base + 2));
                    L = L + mul(tp, ms.emission);
                    tp = mul(tp, ms.radiance * (fabsf(dot(f.normal, ms.outgoing)) / ms.pdf));
                    new_o = nudge(o + (d * h.x), ms.outgoing);
                    new_d = ms.outgoing;
                    if (depth > J.rr_depth || nearly_zero(tp)) {
                        float rv = uniform01(key, base + 3);
                        float lum = luminance(tp);
                        float prob =
                            depth > J.rr_aggr ? clamped_lerp(0.10f, 0.75f, lum) : clamped_lerp(0.25f, 1.00f, lum);
                        tp = rv < prob ? tp / prob : v3zero();
                    }
                    alive = !is_zero(tp) && (J.max_depth == 0 || depth + 1 < J.max_depth);
                }
                // A live path carries (throughput, radiance, key) to its next queue entry; a
                // finished one leaves its radiance in its slot, which with the cold record's
                // film position is all the gather reads.
                if (alive) {
                    sa = make_float4(tp.x, tp.y, tp.z, L.x);
                    sb = make_float4(L.y, L.z, hb.z, hb.w);
                } else {
                    s_hot[slot] = make_float4(L.x, L.y, L.z, 0.0f);
                    finished = true;
                    unit = s_cold[slot].x;
                }
            }
            // Finished paths count their unit done: one atomic per unit per warp.  The
            // plan and gather kernels that read the counts and the samples are later
            // launches on the same stream.
            if (__any_sync(0xffffffffu, finished)) {
                unsigned same = __match_any_sync(0xffffffffu, unit);
                if (finished && lane == static_cast<unsigned>(__ffs(same) - 1))
                    atomicAdd(unit_done + unit, static_cast<uint32_t>(__popc(same)));
            }
            push_ray(alive, &c->q[nxt], slot, new_o, new_d, job, depth + 1, sa, sb, nslot, no, nd, nstate, cap);
        }
        __syncthreads();  // sm is reused by the next chunk
    }
}

int grid_for(const void* kernel, int block, size_t smem, uint32_t n) {
    const int sm = device_sm_count();  // of the current device, asked at each launch
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    uint32_t need = (n + block - 1) / block;
    return static_cast<int>(std::max(1u, std::min(need, static_cast<uint32_t>(sm * per_sm))));
}

template <int W, int BS>
gr_status launch_extend(EngineCtl* c, int cur, const DevJob* jobs, const float4* qo, const float4* qd, float4* qh,
                        uint32_t cap, cudaStream_t st) {
    size_t smem = step_stack_smem_bytes(BS);
    if (GR_EXTEND_REFILL > 0) {
        int grid = grid_for(reinterpret_cast<const void*>(k_eng_extend_refill<W, BS>), BS, smem, cap);
        k_eng_extend_refill<W, BS><<<grid, BS, smem, st>>>(c, cur, jobs, qo, qd, qh);
    } else {
        int grid = grid_for(reinterpret_cast<const void*>(k_eng_extend<W, BS>), BS, smem, cap);
        k_eng_extend<W, BS><<<grid, BS, smem, st>>>(c, cur, jobs, qo, qd, qh);
    }
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

template <int W>
gr_status launch_extend_w(uint32_t bs, EngineCtl* c, int cur, const DevJob* jobs, const float4* qo, const float4* qd,
                          float4* qh, uint32_t cap, cudaStream_t st) {
    switch (bs) {
        case 64: return launch_extend<W, 64>(c, cur, jobs, qo, qd, qh, cap, st);
        case 256: return launch_extend<W, 256>(c, cur, jobs, qo, qd, qh, cap, st);
        default: return launch_extend<W, 128>(c, cur, jobs, qo, qd, qh, cap, st);
    }
}

}  // namespace

#define GR_ETRY(expr)                     \
    do {                                  \
        gr_status s__ = (expr);           \
        if (s__ != GR_OK) return s__;     \
    } while (0)

constexpr uint32_t ENGINE_MAX_JOBS = 4096;
constexpr uint32_t ENGINE_MAX_UNITS = 1u << 20;

Engine::~Engine() {
    if (st_) cudaStreamSynchronize(st_);
    if (graph_) cudaGraphExecDestroy(graph_);
    if (h_pinned_) cudaFreeHost(h_pinned_);
    if (st_) cudaStreamDestroy(st_);
}

gr_status Engine::init(const EngineConfig& cfg, cudaStream_t) {
    cfg_ = cfg;
    if (cfg_.width != 2 && cfg_.width != 4 && cfg_.width != 8) {
        set_error("engine: BVH width must be 2, 4 or 8");
        return GR_ERR_INVALID_ARGUMENT;
    }
    if (cfg_.block != 64 && cfg_.block != 128 && cfg_.block != 256) {
        set_error("engine: block size must be 64, 128 or 256");
        return GR_ERR_INVALID_ARGUMENT;
    }
    if (cfg_.capacity < 1024) cfg_.capacity = 1024;
    uint64_t want = cfg_.ring ? cfg_.ring : 2ull * cfg_.capacity + (1u << 22);
    ring_ = 1u << 20;
    while (ring_ < want && ring_ < (1u << 30)) ring_ <<= 1;  // power of two: the slot is a mask
    GR_CUDA_TRY(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    const size_t C = cfg_.capacity;
    auto alloc = [&](DevBuf& b, size_t bytes) -> cudaError_t {
        bytes_ += bytes;
        return b.ensure(bytes);
    };
    GR_CUDA_TRY(alloc(ctl_, sizeof(EngineCtl)));
    GR_CUDA_TRY(alloc(jobs_, ENGINE_MAX_JOBS * sizeof(DevJob)));
    GR_CUDA_TRY(alloc(units_, ENGINE_MAX_UNITS * sizeof(DevUnit)));
    GR_CUDA_TRY(alloc(unit_done_, ENGINE_MAX_UNITS * sizeof(uint32_t)));
    GR_CUDA_TRY(alloc(s_hot_, static_cast<size_t>(ring_) * 16));
    GR_CUDA_TRY(alloc(s_cold_, static_cast<size_t>(ring_) * 16));
    for (int k = 0; k < 2; ++k) {
        GR_CUDA_TRY(alloc(q_slot_[k], C * 4));
        GR_CUDA_TRY(alloc(q_o_[k], C * 16));
        GR_CUDA_TRY(alloc(q_d_[k], C * 16));
        GR_CUDA_TRY(alloc(q_state_[k], C * 32));
    }
    GR_CUDA_TRY(alloc(q_hit_, C * 16));
    GR_CUDA_TRY(cudaMemsetAsync(ctl_.ptr, 0, sizeof(EngineCtl), st_));
    GR_CUDA_TRY(cudaMemsetAsync(unit_done_.ptr, 0, ENGINE_MAX_UNITS * sizeof(uint32_t), st_));
    GR_CUDA_TRY(cudaHostAlloc(reinterpret_cast<void**>(&h_pinned_), 16 * sizeof(uint64_t), cudaHostAllocDefault));
    GR_CUDA_TRY(cudaStreamSynchronize(st_));
    GR_CUDA_TRY(allow_sort_smem(k_eng_shade, sort_smem_bytes(ESBLOCK, ESHADE_PER_THREAD)));
    return record_pair();
}

gr_status Engine::enqueue_iteration(int cur) {
    EngineCtl* c = ctl_.as<EngineCtl>();
    const uint32_t C = cfg_.capacity;
    const int nxt = cur ^ 1;
    k_eng_plan<<<1, 1, 0, st_>>>(c, jobs_.as<DevJob>(), units_.as<DevUnit>(), unit_done_.as<uint32_t>(), C, ring_, cur);
    GR_CUDA_TRY(cudaGetLastError());
    const int ggrid = grid_for(reinterpret_cast<const void*>(k_eng_gather), FILM_THREADS, 0, 1u << 30);
    k_eng_gather<<<ggrid, FILM_THREADS, 0, st_>>>(c, jobs_.as<DevJob>(), units_.as<DevUnit>(),
                                                                   s_hot_.as<float4>(), s_cold_.as<uint4>(), ring_ - 1);
    GR_CUDA_TRY(cudaGetLastError());
    int fgrid = grid_for(reinterpret_cast<const void*>(k_eng_fill), EBLOCK, 0, C);
    k_eng_fill<<<fgrid, EBLOCK, 0, st_>>>(c, jobs_.as<DevJob>(), units_.as<DevUnit>(), ring_ - 1,
                                          s_cold_.as<uint4>(), q_slot_[cur].as<uint32_t>(), q_o_[cur].as<float4>(),
                                          q_d_[cur].as<float4>(), q_state_[cur].as<float4>(), C);
    GR_CUDA_TRY(cudaGetLastError());
    switch (cfg_.width) {
        case 2:
            GR_ETRY(launch_extend_w<2>(cfg_.block, c, cur, jobs_.as<DevJob>(), q_o_[cur].as<float4>(),
                                       q_d_[cur].as<float4>(), q_hit_.as<float4>(), C, st_));
            break;
        case 8:
            GR_ETRY(launch_extend_w<8>(cfg_.block, c, cur, jobs_.as<DevJob>(), q_o_[cur].as<float4>(),
                                       q_d_[cur].as<float4>(), q_hit_.as<float4>(), C, st_));
            break;
        default:
            GR_ETRY(launch_extend_w<4>(cfg_.block, c, cur, jobs_.as<DevJob>(), q_o_[cur].as<float4>(),
                                       q_d_[cur].as<float4>(), q_hit_.as<float4>(), C, st_));
    }
    GR_CUDA_TRY(cudaMemsetAsync(reinterpret_cast<char*>(c) + offsetof(EngineCtl, q) + nxt * sizeof(uint32_t), 0, 4, st_));
    const size_t ssmem = sort_smem_bytes(ESBLOCK, ESHADE_PER_THREAD);
    int sgrid = grid_for(reinterpret_cast<const void*>(k_eng_shade), ESBLOCK, ssmem, C);
    k_eng_shade<<<sgrid, ESBLOCK, ssmem, st_>>>(c, cur, jobs_.as<DevJob>(), unit_done_.as<uint32_t>(),
                                           q_slot_[cur].as<uint32_t>(), q_o_[cur].as<float4>(), q_d_[cur].as<float4>(),
                                           q_hit_.as<float4>(), q_state_[cur].as<float4>(), s_hot_.as<float4>(),
                                           s_cold_.as<uint4>(), q_slot_[nxt].as<uint32_t>(), q_o_[nxt].as<float4>(),
                                           q_d_[nxt].as<float4>(), q_state_[nxt].as<float4>(), C);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

// Captures two iterations (queues 0 -> 1, then 1 -> 0) as one graph.
gr_status Engine::record_pair() {
    cudaGraph_t g = nullptr;
    GR_CUDA_TRY(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
    gr_status s0 = enqueue_iteration(0);
    gr_status s1 = s0 == GR_OK ? enqueue_iteration(1) : s0;
    cudaError_t e = cudaStreamEndCapture(st_, &g);
    if (s1 != GR_OK) {
        if (g) cudaGraphDestroy(g);
        return s1;
    }
    GR_CUDA_TRY(e);
    cudaError_t ie = cudaGraphInstantiate(&graph_, g, 0);
    cudaGraphDestroy(g);
    GR_CUDA_TRY(ie);
    return GR_OK;
}

gr_status Engine::add_job(const DevJob& job, uint32_t first_pass, uint32_t passes, uint32_t& index) {
    if (h_jobs_.size() >= ENGINE_MAX_JOBS) {
        set_error("engine: too many jobs");
        return GR_ERR_BUSY;
    }
    if (job.scene.width != cfg_.width) {
        set_error("engine: every scene in one engine must have the engine's BVH width");
        return GR_ERR_INVALID_ARGUMENT;
    }
    if (static_cast<uint64_t>(job.npix) * 2 > ring_) {
        set_error("engine: image too large for the path ring");
        return GR_ERR_INVALID_ARGUMENT;
    }
    index = static_cast<uint32_t>(h_jobs_.size());
    h_jobs_.push_back(job);
    GR_CUDA_TRY(cudaMemcpyAsync(jobs_.as<DevJob>() + index, &h_jobs_.back(), sizeof(DevJob), cudaMemcpyHostToDevice,
                                st_));
    std::vector<std::pair<uint32_t, uint32_t>> u;
    for (uint32_t k = 0; k < passes; ++k) u.emplace_back(index, first_pass + k);
    if (!u.empty()) return append_units(u);
    return GR_OK;
}

gr_status Engine::append_units(const std::vector<std::pair<uint32_t, uint32_t>>& units) {
    if (h_units_.size() + units.size() > ENGINE_MAX_UNITS) {
        set_error("engine: too many units");
        return GR_ERR_BUSY;
    }
    uint64_t prefix = 0;
    if (!h_units_.empty()) prefix = h_units_.back().prefix + h_units_.back().npix;
    size_t first = h_units_.size();
    for (auto& pu : units) {
        DevUnit U;
        U.prefix = prefix;
        U.job = pu.first;
        U.pass = pu.second;
        U.npix = h_jobs_[pu.first].npix;
        U.pad = 0;
        prefix += U.npix;
        h_units_.push_back(U);
    }
    GR_CUDA_TRY(cudaMemcpyAsync(units_.as<DevUnit>() + first, h_units_.data() + first, units.size() * sizeof(DevUnit),
                                cudaMemcpyHostToDevice, st_));
    // The kernels read units_count / paths_total from the control block.  Updating them
    // from the host is stream-ordered after every launched iteration.
    uint32_t count = static_cast<uint32_t>(h_units_.size());
    unsigned long long total = prefix;
    h_pinned_[6] = count;
    h_pinned_[7] = total;
    GR_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char*>(ctl_.ptr) + offsetof(EngineCtl, units_count), &h_pinned_[6],
                                4, cudaMemcpyHostToDevice, st_));
    GR_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char*>(ctl_.ptr) + offsetof(EngineCtl, paths_total), &h_pinned_[7],
                                8, cudaMemcpyHostToDevice, st_));
    GR_CUDA_TRY(cudaStreamSynchronize(st_));
    return GR_OK;
}

gr_status Engine::reset() {
    GR_CUDA_TRY(cudaStreamSynchronize(st_));
    size_t used = h_units_.size();
    GR_CUDA_TRY(cudaMemsetAsync(ctl_.ptr, 0, sizeof(EngineCtl), st_));
    if (used) GR_CUDA_TRY(cudaMemsetAsync(unit_done_.ptr, 0, used * sizeof(uint32_t), st_));
    GR_CUDA_TRY(cudaStreamSynchronize(st_));
    h_jobs_.clear();
    h_units_.clear();
    last_ctl_ = EngineCtl{};
    return GR_OK;
}

gr_status Engine::set_flush_unit(uint32_t unit) {
    h_pinned_[12] = unit;
    // Ordered before the next run's replays on the same stream; the pinned word is not
    // written again before that run has synchronised the stream.
    GR_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char*>(ctl_.ptr) + offsetof(EngineCtl, flush_unit), &h_pinned_[12],
                                4, cudaMemcpyHostToDevice, st_));
    return GR_OK;
}

gr_status Engine::cancel_job(uint32_t j) {
    if (j >= h_jobs_.size()) {
        set_error("engine: no such job");
        return GR_ERR_NOT_FOUND;
    }
    h_jobs_[j].live = 0;
    GR_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char*>(jobs_.as<DevJob>() + j) + offsetof(DevJob, live),
                                &h_jobs_[j].live, 4, cudaMemcpyHostToDevice, st_));
    GR_CUDA_TRY(cudaStreamSynchronize(st_));
    return GR_OK;
}

gr_status Engine::run(uint32_t max_pairs, bool& done, uint32_t stop_at_unit) {
    done = false;
    // Replays graph pairs; the done flag and the oldest ungathered unit are copied back
    // after each replay and read one replay behind (the next replay is already queued,
    // so the GPU does not wait for the host).  Replays after completion are empty
    // iterations.
    cudaEvent_t ev[4];
    for (auto& e : ev) GR_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    struct Free {
        cudaEvent_t* e;
        ~Free() {
            for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]);
        }
    } fr{ev};
    const char* done_ptr = reinterpret_cast<const char*>(ctl_.ptr) + offsetof(EngineCtl, done);
    const char* glo_ptr = reinterpret_cast<const char*>(ctl_.ptr) + offsetof(EngineCtl, g_lo);
    // Progress guard: every 256 replays the traced-ray / gathered counters must have
    // moved.
    unsigned long long last_rays = ~0ull;
    uint32_t launched = 0;
    uint32_t last_glo = ~0u;
    for (uint32_t k = 0; k < max_pairs; ++k) {
        if (k && (k & 255) == 0) {
            EngineCtl c;
            GR_CUDA_TRY(cudaStreamSynchronize(st_));
            GR_CUDA_TRY(cudaMemcpy(&c, ctl_.ptr, sizeof(EngineCtl), cudaMemcpyDeviceToHost));
            if (c.done) break;
            if (c.rays == last_rays && c.g_lo == last_glo) {
                set_error("engine: no progress over 256 iterations");
                return GR_ERR_INTERNAL;
            }
            last_rays = c.rays;
            last_glo = c.g_lo;
        }
        GR_CUDA_TRY(cudaGraphLaunch(graph_, st_));
        ++launched;
        h_pinned_[k & 3] = 0;
        h_pinned_[8 + (k & 3)] = 0;
        GR_CUDA_TRY(cudaMemcpyAsync(&h_pinned_[k & 3], done_ptr, 4, cudaMemcpyDeviceToHost, st_));
        GR_CUDA_TRY(cudaMemcpyAsync(&h_pinned_[8 + (k & 3)], glo_ptr, 4, cudaMemcpyDeviceToHost, st_));
        GR_CUDA_TRY(cudaEventRecord(ev[k & 3], st_));
        if (k >= 1) {
            GR_CUDA_TRY(cudaEventSynchronize(ev[(k - 1) & 3]));
            if (h_pinned_[(k - 1) & 3]) break;
            if (h_pinned_[8 + ((k - 1) & 3)] >= stop_at_unit) break;
        }
    }
    GR_CUDA_TRY(cudaStreamSynchronize(st_));
    EngineCtl& c = last_ctl_;
    GR_CUDA_TRY(cudaMemcpy(&c, ctl_.ptr, sizeof(EngineCtl), cudaMemcpyDeviceToHost));
    last_pairs_ = launched;
    done = c.done != 0;
    last_rays_ = c.rays;
    if (c.err == 2) {
        set_error("engine: traversal step budget exceeded");
        return GR_ERR_TIMEOUT;
    }
    if (c.err) {
        set_error("engine: traversal stack bound exceeded");
        return GR_ERR_STACK_OVERFLOW;
    }
#if GR_CHECKED
    bool bad = false;
    GR_CUDA_TRY(take_bad_index(bad));
    if (bad) {
        set_error("engine: a queue index was out of range (checked build)");
        return GR_ERR_INTERNAL;
    }
#endif
    return GR_OK;
}

gr_status Engine::read_ctl(EngineCtl& c) {
    GR_CUDA_TRY(cudaStreamSynchronize(st_));
    GR_CUDA_TRY(cudaMemcpy(&c, ctl_.ptr, sizeof(EngineCtl), cudaMemcpyDeviceToHost));
    return GR_OK;
}

gr_status Engine::unit_done_counts(std::vector<uint32_t>& done) {
    done.resize(h_units_.size());
    if (done.empty()) return GR_OK;
    GR_CUDA_TRY(cudaStreamSynchronize(st_));
    GR_CUDA_TRY(cudaMemcpy(done.data(), unit_done_.ptr, done.size() * 4, cudaMemcpyDeviceToHost));
    return GR_OK;
}

DevJob make_job(gr_scene* scene, const gr_camera& cam, const gr_render_params& p, uint32_t width, uint32_t height,
                float4* film) {
    DevJob j;
    std::memset(&j, 0, sizeof(j));
    j.scene = scene->dev;
    j.cam = make_camera(cam);
    j.film = film;
    j.seed = p.seed;
    j.width = width;
    j.height = height;
    j.npix = width * height;
    j.display = p.integrator == GR_INTEGRATOR_DISPLAY_COLOR ? 1 : 0;
    j.max_depth = j.display ? 1 : p.max_depth;
    j.rr_depth = p.rr_depth;
    j.rr_aggr = p.rr_aggressive_depth;
    j.live = 1;
    return j;
}

}  // namespace gr
