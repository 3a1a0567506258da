// Pieces shared by the wavefront integrators (pt.cu, bdpt.cu): the extension kernel
// over a compacted ray queue, the warp-aggregated queue push and grid sizing.
#pragma once

#include <algorithm>
#include <cstdlib>

#include "runtime.hpp"
#include "shade_sort.cuh"
#include "traverse.cuh"


namespace gr {
namespace {

constexpr int BLOCK = 128;

// Shading kernels are register-heavy (the Disney mixture); asking for 6 resident blocks
// of 128 threads caps them at 85 registers, which measured 3% faster on the bench
// workload than the uncapped 96 (occupancy 31% -> 37%).  GR_SHADE_MIN_BLOCKS overrides.
#ifndef GR_SHADE_MIN_BLOCKS
#define GR_SHADE_MIN_BLOCKS 6
#endif
#define GR_SHADE_BOUNDS __launch_bounds__(BLOCK, GR_SHADE_MIN_BLOCKS)

// Closest hit for every queued ray: a grid-stride loop over the device-side count, so
// launches never depend on a host read of the queue length.  Each thread traverses one
// ray at a time (trace_ray: the step functions and the shared/local hybrid stack); a ray
// that needs more steps than the scene's budget is abandoned and flagged (err = 2).
// GR_EXTEND_MIN_BLOCKS caps registers for that many resident blocks per SM (0: uncapped).
#ifndef GR_EXTEND_MIN_BLOCKS
#define GR_EXTEND_MIN_BLOCKS 0
#endif
#if GR_EXTEND_MIN_BLOCKS > 0
#define GR_EXTEND_BOUNDS __launch_bounds__(BLOCK, GR_EXTEND_MIN_BLOCKS)
#else
#define GR_EXTEND_BOUNDS __launch_bounds__(BLOCK)
#endif

// one_origin: every ray of the queue starts at q_o[0] (the path tracer's camera rays:
// one pinhole origin, stored once).
template <int W, bool COUNT>
__global__ void GR_EXTEND_BOUNDS k_extend(DeviceScene s, const uint32_t* __restrict__ count,
                                                     const float4* __restrict__ q_o, const float4* __restrict__ q_d,
                                                     float4* __restrict__ q_hit, int* err,
                                                     unsigned long long* rays, bool one_origin) {
    extern __shared__ unsigned char smem[];
    int2 spill[MAX_STACK - SMEM_STACK];
    const StackView stk = thread_stack(smem, spill);
    const uint32_t n = *count;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(rays, static_cast<unsigned long long>(n));
    uint32_t counts[2] = {0, 0};
    auto trace = [&](uint32_t q) {
        float4 o4 = q_o[one_origin ? 0 : q], d4 = q_d[q];
        TraceResult r = trace_ray<W, false, COUNT>(s, V3{o4.x, o4.y, o4.z}, V3{d4.x, d4.y, d4.z}, FLT_MAX, stk, err,
                                                   err + 1, q, counts);
        q_hit[q] = make_float4(r.t, __int_as_float(r.k), r.u, r.v);
    };
#if GR_EXTEND_SORT
    // Each block traces its chunk of the queue grouped by direction (octant, dominant axis).
    const SortView sv =
        sort_view<BLOCK, GR_EXTEND_SORT>(smem + static_cast<size_t>(SMEM_STACK) * BLOCK * (sizeof(int32_t) + sizeof(float)));
    const uint32_t per = chunk_per_thread<BLOCK, GR_EXTEND_SORT>(n, gridDim.x);
    const uint32_t chunk = BLOCK * per;
    for (uint32_t c0 = blockIdx.x * chunk; c0 < n; c0 += gridDim.x * chunk) {
        const uint32_t cn = min(chunk, n - c0);
        sort_chunk<BLOCK, GR_EXTEND_SORT>(sv, cn, per, [&](uint32_t i) {
            float4 d = q_d[c0 + i];
            float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
            uint32_t dom = ax >= ay && ax >= az ? 0u : (ay >= az ? 1u : 2u);
            uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
            return oct * 3u + dom;
        });
        for (uint32_t e = 0; e < per; ++e) {
            uint32_t i = e * BLOCK + threadIdx.x;
            if (i < cn) trace(c0 + sv.order[i]);
        }
        __syncthreads();  // sv is reused by the next chunk
    }
#else
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) trace(q);
#endif
    if (COUNT && (counts[0] | counts[1])) {
        atomicAdd(rays + (CNT_NODES - CNT_RAYS) / 2, static_cast<unsigned long long>(counts[0]));
        atomicAdd(rays + (CNT_PRIMS - CNT_RAYS) / 2, static_cast<unsigned long long>(counts[1]));
    }
}

// Refilling variant (GR_EXTEND_REFILL = k > 0): a warp keeps its lanes busy across rays.
// Each iteration every busy lane takes one traversal step; when at least k lanes are
// idle, the warp takes that many rays from a global counter (one atomic) and hands them
// to its idle lanes.  So a lane whose ray ended early starts another one, instead of
// idling until the warp's longest ray ends.
// Every warp intrinsic runs where control flow is warp-uniform: the loop's iterations
// are the same for all lanes, the refill condition depends on ballot results and on the
// fetched base only, and the loop ends on a ballot.  It terminates: an iteration either
// steps a busy lane (each ray has the scene's step budget, and each ray is handed out
// once), or finds every lane idle, refills and gets rays or learns that none are left.
template <int W, bool COUNT>
__global__ void GR_EXTEND_BOUNDS k_extend_refill(DeviceScene s, const uint32_t* __restrict__ count,
                                                 const float4* __restrict__ q_o, const float4* __restrict__ q_d,
                                                 float4* __restrict__ q_hit, int* err, unsigned long long* rays,
                                                 uint32_t* fetch, bool one_origin) {
    extern __shared__ unsigned char smem[];
    int2 spill[MAX_STACK - SMEM_STACK];
    const StackView stk = thread_stack(smem, spill);
    const uint32_t n = *count;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(rays, static_cast<unsigned long long>(n));
    const unsigned lane = threadIdx.x & 31u;
    const unsigned below = (1u << lane) - 1u;
    const uint32_t budget = s.step_budget;
    uint32_t counts[2] = {0, 0};
    TravState t;
    uint32_t q = 0, steps = 0;
    bool busy = false, exhausted = false;
    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, !busy);
        if (!exhausted && __popc(idle) >= (GR_EXTEND_REFILL > 32 ? 32 : GR_EXTEND_REFILL)) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(fetch, static_cast<uint32_t>(__popc(idle)));
            base = __shfl_sync(0xffffffffu, base, 0);
            exhausted = static_cast<uint64_t>(base) + __popc(idle) >= n;
            if (!busy) {
                const uint32_t mine = base + __popc(idle & below);
                if (mine < n) {
                    float4 o4 = q_o[one_origin ? 0u : mine], d4 = q_d[mine];
                    trav_init(t, V3{o4.x, o4.y, o4.z}, V3{d4.x, d4.y, d4.z}, FLT_MAX);
                    q = mine;
                    steps = 0;
                    busy = true;
                }
            }
        }
        // No lane busy only after a refill that found no ray left (a warp with every lane
        // idle always refills while rays remain).
        if (__ballot_sync(0xffffffffu, busy) == 0u) break;
        if (busy) {
            bool done = trav_step<W, false, COUNT>(s, t, stk, err, counts);
            if (!done && ++steps > budget) {
                atomicExch(err, 2);
                atomicExch(err + 1, static_cast<int>(q));
                t.hit = -1;
                done = true;
            }
            if (done) {
                q_hit[q] = make_float4(t.closest, __int_as_float(t.hit), t.hu, t.hv);
                busy = false;
            }
        }
    }
    if (COUNT && (counts[0] | counts[1])) {
        atomicAdd(rays + (CNT_NODES - CNT_RAYS) / 2, static_cast<unsigned long long>(counts[0]));
        atomicAdd(rays + (CNT_PRIMS - CNT_RAYS) / 2, static_cast<unsigned long long>(counts[1]));
    }
}

// Appends this lane's ray to the next queue with one atomic per warp (ballot + popc).
// Every lane of the warp must call it (warp-uniform trip counts).
GR_D void push_warp(bool alive, uint32_t* count_out, uint32_t slot, V3 o, V3 d, uint32_t* __restrict__ nslot,
                    float4* __restrict__ no, float4* __restrict__ nd, uint32_t cap) {
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
    }
}

// Blocks of `block` threads for n items: every block the device can hold at once (SMs x
// resident blocks per SM, asked of the current device at each launch), or fewer when n
// needs fewer.
template <class K>
int resident_grid(K kernel, size_t smem, uint32_t n, int block = BLOCK) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const int sm = device_sm_count();
    uint32_t need = (n + block - 1) / block;
    uint32_t cap = static_cast<uint32_t>(sm * per_sm);
    return static_cast<int>(std::max(1u, std::min(need, cap)));
}

// `fetch`: a counter of the refilling kernel, zeroed here before each launch.
template <int W, bool COUNT>
gr_status extend_launch(const DeviceScene& s, uint32_t cap_n, const uint32_t* count, const float4* qo,
                        const float4* qd, float4* qh, int* err, unsigned long long* rays, uint32_t* fetch,
                        cudaStream_t st, bool one_origin) {
    if (GR_EXTEND_REFILL > 0) {
        size_t smem = step_stack_smem_bytes(BLOCK);
        GR_CUDA_TRY(cudaMemsetAsync(fetch, 0, sizeof(uint32_t), st));
        int grid = resident_grid(k_extend_refill<W, COUNT>, smem, cap_n);
        k_extend_refill<W, COUNT><<<grid, BLOCK, smem, st>>>(s, count, qo, qd, qh, err, rays, fetch, one_origin);
        return GR_OK;
    }
    size_t smem = step_stack_smem_bytes(BLOCK) + (GR_EXTEND_SORT ? sort_smem_bytes(BLOCK, GR_EXTEND_SORT) : 0);
    int grid = resident_grid(k_extend<W, COUNT>, smem, cap_n);
    k_extend<W, COUNT><<<grid, BLOCK, smem, st>>>(s, count, qo, qd, qh, err, rays, one_origin);
    return GR_OK;
}

// one_origin: every ray of the queue starts at qo[0] (see k_extend).
gr_status extend_any(const DeviceScene& s, bool count_traversal, uint32_t cap_n, const uint32_t* count,
                     const float4* qo, const float4* qd, float4* qh, int* err, unsigned long long* rays,
                     uint32_t* fetch, cudaStream_t st, bool one_origin) {
    const bool o1 = one_origin;
    if (count_traversal) {
        switch (s.width) {
            case 2: return extend_launch<2, true>(s, cap_n, count, qo, qd, qh, err, rays, fetch, st, o1);
            case 4: return extend_launch<4, true>(s, cap_n, count, qo, qd, qh, err, rays, fetch, st, o1);
            default: return extend_launch<8, true>(s, cap_n, count, qo, qd, qh, err, rays, fetch, st, o1);
        }
    }
    switch (s.width) {
        case 2: return extend_launch<2, false>(s, cap_n, count, qo, qd, qh, err, rays, fetch, st, o1);
        case 4: return extend_launch<4, false>(s, cap_n, count, qo, qd, qh, err, rays, fetch, st, o1);
        default: return extend_launch<8, false>(s, cap_n, count, qo, qd, qh, err, rays, fetch, st, o1);
    }
}

}  // namespace
}  // namespace gr
