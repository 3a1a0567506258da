// Film accumulation, resolve and EXR packing.
//
// Film::report_samples (render/film.rs:78-114) splats each sample, serially and in
// sample order, over the pixels within 2 px of its jittered position with a Mitchell
// weight.  Samples are jittered at most 2 px from their own pixel, so a pixel only
// receives samples from pixels at most 4 away.  The gather below gives each thread
// one destination pixel; a 16x16 tile stages the samples of its 24x24 neighbourhood
// (footprint precomputed) in shared memory, and every pixel adds its contributors in
// increasing sample index (rows, then columns), pass after pass.  That is the order of
// the reference's serial loop, so the sums are bit-identical to it, with no atomics.
#include "runtime.hpp"

namespace gr {

namespace {

constexpr int TILE = 16;
constexpr int HALO = 4;
constexpr int SPAN = TILE + 2 * HALO;  // 24

// core/math.rs:92-123 (B = C = 1/3)
GR_D float mitchell1(float x) {
    const float B = 1.0f / 3.0f;
    const float C = 1.0f / 3.0f;
    float twox = fabsf(2.0f * x);
    if (twox > 1.0f) {
        return ((-B - 6.0f * C) * (twox * twox * twox) + (6.0f * B + 30.0f * C) * (twox * twox) +
                (-12.0f * B - 48.0f * C) * twox + (8.0f * B + 24.0f * C)) *
               (1.0f / 6.0f);
    }
    return ((12.0f - 9.0f * B - 6.0f * C) * (twox * twox * twox) + (-18.0f + 12.0f * B + 6.0f * C) * (twox * twox) +
            (6.0f - 2.0f * B)) *
           (1.0f / 6.0f);
}

struct StagedSample {
    float cd, rd;  // col_discr, row_discr
    short minc, maxc, minr, maxr;
    float r, g, b;
};

__global__ void __launch_bounds__(TILE* TILE) k_film_gather(const float2* __restrict__ st,
                                                           const float4* __restrict__ color, uint32_t width,
                                                           uint32_t height, uint32_t passes, float4* film) {
    __shared__ StagedSample sm[SPAN * SPAN];
    const int ox = blockIdx.x * TILE, oy = blockIdx.y * TILE;
    const int tx = threadIdx.x % TILE, ty = threadIdx.x / TILE;
    const int x = ox + tx, y = oy + ty;
    const bool inside = x < static_cast<int>(width) && y < static_cast<int>(height);
    const float wf = static_cast<float>(width), hf = static_cast<float>(height);
    const long long last_col = static_cast<long long>(width) - 1, last_row = static_cast<long long>(height) - 1;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (inside) acc = film[static_cast<size_t>(y) * width + x];
    const size_t npix = static_cast<size_t>(width) * height;
    for (uint32_t pass = 0; pass < passes; ++pass) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < SPAN * SPAN; idx += TILE * TILE) {
            int sr = oy - HALO + idx / SPAN, sc = ox - HALO + idx % SPAN;
            StagedSample e;
            e.minc = 1;
            e.maxc = 0;  // empty footprint
            e.minr = 1;
            e.maxr = 0;
            e.cd = e.rd = 0.0f;
            e.r = e.g = e.b = 0.0f;
            if (sr >= 0 && sc >= 0 && sr < static_cast<int>(height) && sc < static_cast<int>(width)) {
                size_t i = pass * npix + static_cast<size_t>(sr) * width + sc;
                float2 s = st[i];
                float4 c = color[i];
                // film.rs:82-97
                float col_cont = lerp(0.0f, wf, 0.5f * (s.x + 1.0f));
                float row_cont = lerp(0.0f, hf, 0.5f * (s.y + 1.0f));
                float cd = col_cont - 0.5f, rd = row_cont - 0.5f;
                long long mnc = static_cast<long long>(ceilf(cd - 2.0f));
                long long mxc = static_cast<long long>(floorf(cd + 2.0f));
                long long mnr = static_cast<long long>(ceilf(rd - 2.0f));
                long long mxr = static_cast<long long>(floorf(rd + 2.0f));
                mnc = mnc < 0 ? 0 : (mnc > last_col ? last_col : mnc);
                mxc = mxc < 0 ? 0 : (mxc > last_col ? last_col : mxc);
                mnr = mnr < 0 ? 0 : (mnr > last_row ? last_row : mnr);
                mxr = mxr < 0 ? 0 : (mxr > last_row ? last_row : mxr);
                e.cd = cd;
                e.rd = rd;
                // Relative to the tile origin; footprints never exceed +-4 px of the source.
                e.minc = static_cast<short>(mnc - ox);
                e.maxc = static_cast<short>(mxc - ox);
                e.minr = static_cast<short>(mnr - oy);
                e.maxr = static_cast<short>(mxr - oy);
                e.r = c.x;
                e.g = c.y;
                e.b = c.z;
            }
            sm[idx] = e;
        }
        __syncthreads();
        if (!inside) continue;
#pragma unroll 1
        for (int dy = 0; dy <= 2 * HALO; ++dy) {
#pragma unroll
            for (int dx = 0; dx <= 2 * HALO; ++dx) {
                const StagedSample& e = sm[(ty + dy) * SPAN + (tx + dx)];
                if (tx >= e.minc && tx <= e.maxc && ty >= e.minr && ty <= e.maxr) {
                    float w = mitchell1((static_cast<float>(x) - e.cd) / 2.0f) *
                              mitchell1((static_cast<float>(y) - e.rd) / 2.0f);
                    acc.x = acc.x + e.r * w;
                    acc.y = acc.y + e.g * w;
                    acc.z = acc.z + e.b * w;
                    acc.w += w;
                }
            }
        }
    }
    if (inside) film[static_cast<size_t>(y) * width + x] = acc;
}

__global__ void k_resolve(const float4* __restrict__ film, uint32_t n, float* rgb) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = film[i];
    rgb[3 * i] = p.x / p.w;
    rgb[3 * i + 1] = p.y / p.w;
    rgb[3 * i + 2] = p.z / p.w;
}

// ExrWriter::write_channels (render/exr.rs:138-166): per scanline y, the int32 line
// number, the uint32 byte count and the B, G, R planes of film row height - y - 1.
__global__ void k_exr_pack(const float4* __restrict__ film, uint32_t width, uint32_t height, unsigned char* out) {
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
    float4 p = film[static_cast<size_t>(height - y - 1) * width + i];
    float v[3] = {p.x / p.w, p.y / p.w, p.z / p.w};
    float* planes = reinterpret_cast<float*>(l + 8);  // 8 + 12 * width keeps 4-byte alignment
    planes[i] = v[2];
    planes[width + i] = v[1];
    planes[2 * width + i] = v[0];
}

}  // namespace

gr_status film_gather(const float2* st, const float4* color, uint32_t width, uint32_t height, uint32_t passes,
                      float4* film, cudaStream_t s) {
    dim3 grid((width + TILE - 1) / TILE, (height + TILE - 1) / TILE);
    k_film_gather<<<grid, TILE * TILE, 0, s>>>(st, color, width, height, passes, film);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

gr_status film_resolve(const float4* film, uint32_t n, float* rgb, cudaStream_t s) {
    k_resolve<<<(n + 255) / 256, 256, 0, s>>>(film, n, rgb);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

gr_status film_exr_pack(const float4* film, uint32_t width, uint32_t height, unsigned char* out, size_t,
                        cudaStream_t s) {
    dim3 grid((width + 127) / 128, height);
    k_exr_pack<<<grid, 128, 0, s>>>(film, width, height, out);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

}  // namespace gr
