// Film accumulation (the deterministic tile gather of film_gather.cuh, pass after pass),
// resolve and EXR packing.
#include <cstdlib>

#include "film_gather.cuh"
#include "runtime.hpp"

namespace gr {

namespace {

// Passes per work item of the chunked gather.
constexpr uint32_t FILM_CHUNK_PASSES = 8;
// Polls an item makes for its tile's previous chunk (an L2 atomic and a 0.1 us sleep
// each): about 2 s.
constexpr uint32_t FILM_WAIT_LIMIT = 1u << 21;
// GR_FILM_WAIT_TEST=1 (tests only): the chunked gather starts its item counter past the
// first chunk, whose items then never run, so every later item's wait runs out (after
// FILM_WAIT_TEST_LIMIT polls) and the render reports it.  No fault, and every wait ends.
constexpr uint32_t FILM_WAIT_TEST_LIMIT = 1u << 12;
constexpr int FILM_ERR_WAIT = 3;  // error word: a wait ran out

__global__ void k_film_set_word(uint32_t* w, uint32_t v) { *w = v; }

// One block per tile, all passes.
__global__ void __launch_bounds__(FILM_THREADS, GR_FILM_BLOCKS_PER_SM) k_film_gather(const float2* __restrict__ st,
                                                              const float4* __restrict__ color, uint32_t width,
                                                              uint32_t height, uint32_t passes, float4* film) {
    __shared__ StagedSample sm;
    const int ox = blockIdx.x * FILM_TILE_W, oy = blockIdx.y * FILM_TILE_H;
    const int x = ox + threadIdx.x % FILM_TILE_W, y = oy + threadIdx.x / FILM_TILE_W;
    const bool inside = x < static_cast<int>(width) && y < static_cast<int>(height);
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (inside) acc = film[static_cast<size_t>(y) * width + x];
    const size_t npix = static_cast<size_t>(width) * height;
    gather_passes(sm, width, height, ox, oy, acc, passes,
                  [&](uint32_t pass) { return LinearSamples{st, color, pass * npix, width}; });
    if (inside) film[static_cast<size_t>(y) * width + x] = acc;
}

// Ordered chunks: work item i is passes [c * 8, c * 8 + 8) of tile i % ntiles, c = i /
// ntiles.  With one block per tile, all passes, a launch of T tiles on S resident blocks
// runs ceil(T / S) rounds of whole tiles; eight-pass items shrink the idle last round
// eightfold.  A pixel's sum stays in pass order: an item starts from the film its tile's
// previous chunk stored, once that chunk's flag (sched[1 + tile]) says so.  Items are
// taken in increasing order from a counter (sched[0]), so the item waited for went to a
// block that is already running and waits only for smaller items: every wait ends.  A
// wait is still bounded; one that runs out sets *err and skips its item.
__global__ void __launch_bounds__(FILM_THREADS, GR_FILM_BLOCKS_PER_SM)
    k_film_gather_chunked(const float2* __restrict__ st, const float4* __restrict__ color, uint32_t width,
                          uint32_t height, uint32_t passes, float4* film, uint32_t* sched, int* err,
                          uint32_t wait_limit) {
    __shared__ StagedSample sm;
    __shared__ uint32_t s_item;
    __shared__ int s_skip;
    const uint32_t tiles_x = film_tiles_x(width), ntiles = tiles_x * film_tiles_y(height);
    const uint32_t items = ntiles * ((passes + FILM_CHUNK_PASSES - 1) / FILM_CHUNK_PASSES);
    const size_t npix = static_cast<size_t>(width) * height;
    uint32_t* flags = sched + 1;
    for (;;) {
        if (threadIdx.x == 0) {
            uint32_t item = atomicAdd(sched, 1u);
            int skip = 0;
            if (item < items && item >= ntiles) {  // wait for chunk c - 1 of the tile
                const uint32_t c = item / ntiles, tile = item - c * ntiles;
                uint32_t polls = 0;
                while (atomicAdd(flags + tile, 0u) < c) {
                    if (++polls > wait_limit) {
                        atomicExch(err, FILM_ERR_WAIT);
                        skip = 1;
                        break;
                    }
                    __nanosleep(100);
                }
                __threadfence();  // the stored film is read after the flag
            }
            s_item = item;
            s_skip = skip;
        }
        __syncthreads();
        const uint32_t item = s_item;
        const int skip = s_skip;
        if (item >= items) return;  // uniform: every thread read the same item
        const uint32_t c = item / ntiles, tile = item - c * ntiles;
        const int ox = static_cast<int>((tile % tiles_x) * FILM_TILE_W);
        const int oy = static_cast<int>((tile / tiles_x) * FILM_TILE_H);
        const int x = ox + threadIdx.x % FILM_TILE_W, y = oy + threadIdx.x / FILM_TILE_W;
        const bool inside = x < static_cast<int>(width) && y < static_cast<int>(height);
        if (!skip) {
            float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            float4* px = film + static_cast<size_t>(y) * width + x;
            if (inside) acc = __ldcg(px);  // from L2: another SM may have stored it
            const uint32_t p0 = c * FILM_CHUNK_PASSES, np = min(FILM_CHUNK_PASSES, passes - p0);
            gather_passes(sm, width, height, ox, oy, acc, np, [&](uint32_t k) {
                return LinearSamples{st, color, static_cast<size_t>(p0 + k) * npix, width};
            });
            if (inside) __stcg(px, acc);
            __threadfence();  // this thread's film store before the tile's flag
        }
        __syncthreads();  // every store is fenced; sm and s_item are free again
        if (threadIdx.x == 0 && !skip) atomicExch(flags + tile, c + 1);
    }
}

// accum / weight, plus splat * scale (light-tracing extension) when splat is not null.
GR_D V3 resolved(const float4* __restrict__ film, const float4* __restrict__ splat, float scale, size_t i) {
    float4 p = film[i];
    V3 v = V3{p.x / p.w, p.y / p.w, p.z / p.w};
    if (splat) {
        float4 q = splat[i];
        v = v + V3{q.x, q.y, q.z} * scale;
    }
    return v;
}

__global__ void k_resolve(const float4* __restrict__ film, const float4* __restrict__ splat, float scale, uint32_t n,
                          float* rgb) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 v = resolved(film, splat, scale, i);
    rgb[3 * i] = v.x;
    rgb[3 * i + 1] = v.y;
    rgb[3 * i + 2] = v.z;
}

// Film::pixels as two planes: accum (3 floats per pixel) and weight (1 float per pixel).
__global__ void k_film_split(const float4* __restrict__ film, uint32_t n, float* __restrict__ accum,
                             float* __restrict__ weight) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = film[i];
    accum[3 * i] = p.x;
    accum[3 * i + 1] = p.y;
    accum[3 * i + 2] = p.z;
    weight[i] = p.w;
}

// ExrWriter::write_channels (render/exr.rs:138-166): per scanline y, the int32 line
// number, the uint32 byte count and the B, G, R planes of film row height - y - 1.
__global__ void k_exr_pack(const float4* __restrict__ film, const float4* __restrict__ splat, float scale,
                           uint32_t width, uint32_t height, unsigned char* out) {
    uint32_t y = blockIdx.y;
    size_t line = 8 + static_cast<size_t>(width) * 12;
    unsigned char* l = out + y * line;
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int32_t yy = static_cast<int32_t>(y);
        uint32_t bytes = static_cast<uint32_t>(line - 8);
        memcpy(l, &yy, 4);
        memcpy(l + 4, &bytes, 4);
    }
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= width) return;
    V3 r = resolved(film, splat, scale, static_cast<size_t>(height - y - 1) * width + i);
    float v[3] = {r.x, r.y, r.z};
    float* planes = reinterpret_cast<float*>(l + 8);  // 8 + 12 * width keeps 4-byte alignment
    planes[i] = v[2];
    planes[width + i] = v[1];
    planes[2 * width + i] = v[0];
}

}  // namespace

size_t film_sched_words(uint32_t width, uint32_t height) {
    return 1 + static_cast<size_t>(film_tiles_x(width)) * film_tiles_y(height);
}

gr_status film_gather(const float2* st, const float4* color, uint32_t width, uint32_t height, uint32_t passes,
                      float4* film, cudaStream_t s, uint32_t* sched, int* err) {
    if (passes == 0 || width == 0 || height == 0) return GR_OK;
    const uint32_t ntiles = film_tiles_x(width) * film_tiles_y(height);
    int per_sm = 0;
    GR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_film_gather_chunked, FILM_THREADS, 0));
    const uint32_t slots = static_cast<uint32_t>(std::max(1, per_sm * device_sm_count()));
    // Chunks pay off when the tiles fill the resident blocks at least once; a smaller
    // image's chunks would only wait on one another.
    if (sched && err && passes > FILM_CHUNK_PASSES && ntiles >= slots) {
        GR_CUDA_TRY(cudaMemsetAsync(sched, 0, film_sched_words(width, height) * sizeof(uint32_t), s));
        const char* wt = std::getenv("GR_FILM_WAIT_TEST");
        const bool wait_test = wt && std::atoi(wt) > 0;
        if (wait_test) k_film_set_word<<<1, 1, 0, s>>>(sched, ntiles);
        const uint32_t items = ntiles * ((passes + FILM_CHUNK_PASSES - 1) / FILM_CHUNK_PASSES);
        k_film_gather_chunked<<<std::min(items, slots), FILM_THREADS, 0, s>>>(st, color, width, height, passes, film,
                                                                              sched, err,
                                                                              wait_test ? FILM_WAIT_TEST_LIMIT
                                                                                        : FILM_WAIT_LIMIT);
    } else {
        dim3 grid(film_tiles_x(width), film_tiles_y(height));
        k_film_gather<<<grid, FILM_THREADS, 0, s>>>(st, color, width, height, passes, film);
    }
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

gr_status film_resolve(const float4* film, const float4* splat, float splat_scale, uint32_t n, float* rgb,
                       cudaStream_t s) {
    k_resolve<<<(n + 255) / 256, 256, 0, s>>>(film, splat, splat_scale, n, rgb);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

gr_status film_split(const float4* film, uint32_t n, float* accum, float* weight, cudaStream_t s) {
    k_film_split<<<(n + 255) / 256, 256, 0, s>>>(film, n, accum, weight);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

gr_status film_exr_pack(const float4* film, const float4* splat, float splat_scale, uint32_t width, uint32_t height,
                        unsigned char* out, size_t, cudaStream_t s) {
    dim3 grid((width + 127) / 128, height);
    k_exr_pack<<<grid, 128, 0, s>>>(film, splat, splat_scale, width, height, out);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

}  // namespace gr
