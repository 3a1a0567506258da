// Block-local counting sort of a chunk of queue positions by a small bucket id.  The
// shading kernels use it to run coherent warps: a block sorts its chunk of the queue by
// code path (the chosen lobe's type and the material's lobe types) in shared memory,
// then shades the chunk in that order, so a warp runs one lobe sampler and one mixture
// instead of a mix of all of them.  The order only decides which thread handles which
// queue entry; no result depends on it.
#pragma once

#include "common.cuh"
#include "scene.hpp"

namespace gr {

constexpr uint32_t SORT_BUCKETS = 32;

// Most queue entries each thread of a shading block sorts and shades per chunk.  Larger
// chunks give fuller warps per bucket and amortise the sort's barriers; on the
// path-tracer workload 4 -> 8 -> 16 entries per thread measured 937 -> 1011 -> 1070
// Msamples/s.  The entries per thread of a launch are chosen from the queue length
// (chunk_per_thread) so that small queues still spread over every block.
#ifndef GR_SHADE_PER_THREAD
#define GR_SHADE_PER_THREAD 64
#endif
constexpr uint32_t SHADE_PER_THREAD = GR_SHADE_PER_THREAD;
// Entries per thread per chunk of the 768-thread shading blocks (one per SM): 85 at most
// (768 x 85 chunk positions fit 16 bits).  A block sorts its whole chunk (reading every
// entry's hit and key) before it shades it; at 85 per thread the chunks of all SMs (about
// 476 MB of those lines) overflow L2 between the two reads.  On the path-tracer workload
// (102,422 triangles, 1024 x 1024, 64 spp) 16 / 24 / 32 / 40 / 64 / 85 measured shading
// 9.39 (with an L2 prefetch) / 9.08 / 9.10 / 9.43 / 9.69 / 10.32 ms per render.
#ifndef GR_SHADE_BIG_PER
#define GR_SHADE_BIG_PER 32
#endif
constexpr uint32_t SHADE_BIG_PER = GR_SHADE_BIG_PER;
static_assert(SHADE_BIG_PER >= 1 && SHADE_BIG_PER <= 85, "768 x per chunk positions fit 16 bits");

// Rays per thread per chunk when the extension kernels trace their queue grouped by
// direction (octant and dominant axis; 0: no sort).  Measured on the path-tracer
// workload: 8 -> +2.2%; 2, 32 and 64 slower (the barrier per chunk waits for the chunk's
// slowest ray, which outweighs the coherence gained).
#ifndef GR_EXTEND_SORT
#define GR_EXTEND_SORT 8
#endif

// The sort's shared memory (dynamic, sort_smem_bytes(NT, PER) bytes at the start of the
// block's dynamic shared memory): bucket sizes, then per-entry bucket and sorted order.
struct SortView {
    uint32_t* count;  // SORT_BUCKETS: bucket sizes, then running positions
    uint8_t* bucket;
    uint16_t* order;
};

inline size_t sort_smem_bytes(uint32_t nt, uint32_t per) {
    return SORT_BUCKETS * sizeof(uint32_t) + static_cast<size_t>(nt) * per * (sizeof(uint8_t) + sizeof(uint16_t));
}

// Lets `kernel` use `bytes` of dynamic shared memory (needed above 48 KB).  Call it
// before the first launch (and before a graph capture that contains one).
template <class K>
cudaError_t allow_sort_smem(K kernel, size_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

template <uint32_t NT, uint32_t PER>
GR_D SortView sort_view(unsigned char* smem) {
    uint32_t* count = reinterpret_cast<uint32_t*>(smem);
    uint16_t* order = reinterpret_cast<uint16_t*>(count + SORT_BUCKETS);
    uint8_t* bucket = reinterpret_cast<uint8_t*>(order + NT * PER);
    return SortView{count, bucket, order};
}

// Entries per thread for a queue of n entries over `blocks` blocks of NT threads: about
// one chunk per block, at most PER.
template <uint32_t NT, uint32_t PER>
GR_D uint32_t chunk_per_thread(uint32_t n, uint32_t blocks) {
    uint32_t per = (n + blocks * NT - 1) / (blocks * NT);
    return per < 1 ? 1 : (per > PER ? PER : per);
}

// Entries per chunk for a queue of n entries over `blocks` blocks of NT threads taking
// `per` entries per thread: NT * per, or, when the queue cannot give every block NT
// entries (per == 1), a multiple of 32 that spreads it over all blocks, so a short queue
// still runs on every SM.
template <uint32_t NT>
GR_D uint32_t chunk_entries(uint32_t n, uint32_t blocks, uint32_t per) {
    if (per > 1) return NT * per;
    uint32_t c = (n + blocks - 1) / blocks;
    c = (c + 31u) & ~31u;
    return c == 0 ? 32u : (c < NT ? c : NT);
}

// Sorts positions 0..cn-1 (cn <= NT * per, per <= PER) by bucket_of(i) < SORT_BUCKETS
// into sm.order.  Every thread of an NT-thread block must call it with the same cn and
// per.  It ends with a barrier; the caller needs one more before the next call reuses
// `sm`.  Within a bucket the order is unspecified.
template <uint32_t NT, uint32_t PER, class F>
GR_D void sort_chunk(const SortView& sm, uint32_t cn, uint32_t per, F bucket_of) {
    static_assert(NT * PER <= 65536, "chunk positions are 16-bit");
    static_assert(SORT_BUCKETS == 32, "the scan below is one warp");
    const uint32_t tid = threadIdx.x;
    if (tid < SORT_BUCKETS) sm.count[tid] = 0;
    __syncthreads();
    for (uint32_t e = 0; e < per; ++e) {
        uint32_t i = e * NT + tid;
        if (i < cn) {
            uint32_t b = bucket_of(i);
            sm.bucket[i] = static_cast<uint8_t>(b);
            atomicAdd(&sm.count[b], 1u);
        }
    }
    __syncthreads();
    if (tid < 32) {  // exclusive scan of the bucket sizes
        uint32_t c = sm.count[tid], x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (static_cast<int>(tid) >= o) x += y;
        }
        sm.count[tid] = x - c;
    }
    __syncthreads();
    for (uint32_t e = 0; e < per; ++e) {
        uint32_t i = e * NT + tid;
        if (i < cn) sm.order[atomicAdd(&sm.count[sm.bucket[i]], 1u)] = static_cast<uint16_t>(i);
    }
    __syncthreads();
}

// Bucket of a shading entry: 0 when the ray escaped.  Otherwise the code path
// Material::sample_world will take: the type of the lobe it picks from the uniform u0
// (material.rs:151-153) and the material's lobe types, which the mixture's f / pdf loop
// runs through.  Six lobe types use buckets 1-30 (5 each), the lobe set and `salt` (a
// walk kind) choosing among the 5.  Materials of any scene or job with the same lobe
// types share a bucket.
GR_D uint32_t shade_bucket(const DeviceScene& s, int32_t k, float u0, uint32_t salt) {
    if (k < 0) return 0;
    uint32_t prim = __float_as_uint(__ldg(s.prims + 3 * static_cast<size_t>(k)).w);
    const DevMaterial& m = s.materials[__ldg(s.prim_material + prim)];
    const uint32_t nl = static_cast<uint32_t>(m.n_lobes);
    if (nl == 0) return 1;
    const uint32_t r = range_index(u0, nl);
    const uint32_t chosen = static_cast<uint32_t>(m.lobe[r].type);
    return 1 + 5 * (chosen % 6) + ((m.lobe_set + salt) * 0x9E3779B1u >> 16) % 5;
}

}  // namespace gr
