// Deterministic film splat, shared by the per-image render (film.cu) and the engine.
//
// Film::report_samples (render/film.rs:78-114) splats each sample, serially and in
// sample order, over the pixels within 2 px of its jittered position with a Mitchell
// weight.  Samples are jittered at most 2 px from their own pixel, so a pixel only
// receives samples from pixels at most 4 away.  gather_tile gives each thread one
// destination pixel; a 16x16 tile stages the samples of its 24x24 neighbourhood
// (footprint precomputed) in shared memory, and every pixel adds its contributors in
// increasing sample index (rows, then columns).  That is the order of the reference's
// serial loop, so the sums are bit-identical to it, with no atomics.
#pragma once

#include "common.cuh"

namespace gr {

constexpr int FILM_TILE = 16;
constexpr int FILM_HALO = 4;
constexpr int FILM_SPAN = FILM_TILE + 2 * FILM_HALO;  // 24

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

// Adds the samples of one pass to the tile (ox, oy) of `film`.  `src(row, col, st, rgb)`
// loads that pixel's sample: its film position (s, t) and its radiance.  Every thread of
// the block (256 = FILM_TILE^2) must call it; `sm` holds FILM_SPAN^2 entries.
template <class Src>
GR_D void gather_tile(StagedSample* sm, uint32_t width, uint32_t height, int ox, int oy, float4& acc, const Src& src) {
    const int tx = threadIdx.x % FILM_TILE, ty = threadIdx.x / FILM_TILE;
    const int x = ox + tx, y = oy + ty;
    const bool inside = x < static_cast<int>(width) && y < static_cast<int>(height);
    const float wf = static_cast<float>(width), hf = static_cast<float>(height);
    const long long last_col = static_cast<long long>(width) - 1, last_row = static_cast<long long>(height) - 1;
    __syncthreads();
    for (int k = threadIdx.x; k < FILM_SPAN * FILM_SPAN; k += FILM_TILE * FILM_TILE) {
        int sr = oy - FILM_HALO + k / FILM_SPAN, sc = ox - FILM_HALO + k % FILM_SPAN;
        StagedSample e;
        e.minc = 1;
        e.maxc = 0;  // empty footprint
        e.minr = 1;
        e.maxr = 0;
        e.cd = e.rd = 0.0f;
        e.r = e.g = e.b = 0.0f;
        if (sr >= 0 && sc >= 0 && sr < static_cast<int>(height) && sc < static_cast<int>(width)) {
            float2 s;
            V3 c;
            src(static_cast<uint32_t>(sr), static_cast<uint32_t>(sc), s, c);
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
        sm[k] = e;
    }
    __syncthreads();
    if (!inside) return;
#pragma unroll 1
    for (int dy = 0; dy <= 2 * FILM_HALO; ++dy) {
#pragma unroll
        for (int dx = 0; dx <= 2 * FILM_HALO; ++dx) {
            const StagedSample& e = sm[(ty + dy) * FILM_SPAN + (tx + dx)];
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

// Samples of one pass stored linearly: sample (row, col) at base + row * width + col of
// `st` (film position) and `color` (radiance in xyz).
struct LinearSamples {
    const float2* __restrict__ st;
    const float4* __restrict__ color;
    size_t base;
    uint32_t width;
    GR_D void operator()(uint32_t r, uint32_t c, float2& s, V3& rgb) const {
        size_t i = base + static_cast<size_t>(r) * width + c;
        s = st[i];
        float4 v = color[i];
        rgb = V3{v.x, v.y, v.z};
    }
};

}  // namespace gr
