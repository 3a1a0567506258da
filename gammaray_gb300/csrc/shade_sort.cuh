// Block-local counting sort of a chunk of queue positions by a small bucket id.  The
// shading kernels use it to run coherent warps: a block sorts its chunk of the queue by
// (material, chosen lobe) in shared memory, then shades the chunk in that order, so a
// warp runs one material's one lobe sampler instead of a mix of all of them.  The order
// only decides which thread handles which queue entry; no result depends on it.
#pragma once

#include "common.cuh"
#include "scene.hpp"

namespace gr {

constexpr uint32_t SORT_BUCKETS = 32;

template <uint32_t NT, uint32_t PER>
struct SortSmem {
    uint32_t start[SORT_BUCKETS];
    uint16_t order[NT * PER];
};

// Sorts positions 0..cn-1 (cn <= NT * PER) by bucket_of(i) < SORT_BUCKETS into
// sm.order.  Every thread of an NT-thread block must call it.  It ends with a barrier;
// the caller needs one more before the next call reuses `sm`.  Within a bucket the order
// is unspecified.
template <uint32_t NT, uint32_t PER, class F>
GR_D void sort_chunk(SortSmem<NT, PER>& sm, uint32_t cn, F bucket_of) {
    static_assert(NT * PER <= 65536, "chunk positions are 16-bit");
    static_assert(SORT_BUCKETS == 32, "the scan below is one warp");
    const uint32_t tid = threadIdx.x;
    if (tid < SORT_BUCKETS) sm.start[tid] = 0;
    __syncthreads();
    uint32_t bucket[PER], rank[PER];
#pragma unroll
    for (uint32_t e = 0; e < PER; ++e) {
        uint32_t i = e * NT + tid;
        bucket[e] = 0;
        rank[e] = 0;
        if (i < cn) {
            bucket[e] = bucket_of(i);
            rank[e] = atomicAdd(&sm.start[bucket[e]], 1u);
        }
    }
    __syncthreads();
    if (tid < 32) {  // exclusive scan of the bucket counts
        uint32_t c = sm.start[tid], x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (static_cast<int>(tid) >= o) x += y;
        }
        sm.start[tid] = x - c;
    }
    __syncthreads();
#pragma unroll
    for (uint32_t e = 0; e < PER; ++e) {
        uint32_t i = e * NT + tid;
        if (i < cn) sm.order[sm.start[bucket[e]] + rank[e]] = static_cast<uint16_t>(i);
    }
    __syncthreads();
}

// Bucket of a shading entry: 0 when the ray escaped, else a hash of the hit's material,
// of `salt` (a job, a walk kind) and of the lobe Material::sample_world will pick from
// the uniform u0 (material.rs:151-153).
GR_D uint32_t shade_bucket(const DeviceScene& s, int32_t k, float u0, uint32_t salt) {
    if (k < 0) return 0;
    uint32_t prim = __float_as_uint(__ldg(s.prims + 3 * static_cast<size_t>(k)).w);
    uint32_t mat = __ldg(s.prim_material + prim);
    uint32_t nl = static_cast<uint32_t>(s.materials[mat].n_lobes);
    uint32_t r = nl ? range_index(u0, nl) : 0;
    return 1 + ((salt * 0x9E3779B1u) ^ (mat * MAX_LOBES + r)) % (SORT_BUCKETS - 1);
}

}  // namespace gr
