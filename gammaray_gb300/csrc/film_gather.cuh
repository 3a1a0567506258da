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

// A tile's staged samples (structure of arrays, FILM_SPAN^2 of them) and, per tile pixel,
// an 81-bit mask of the samples in its 9x9 neighbourhood whose footprint covers it (bit
// dy * 9 + dx for the sample dy rows and dx columns below / right of the neighbourhood's
// corner).  Visiting set bits in increasing order is visiting contributors in
// increasing sample index, the reference's order.
constexpr int FILM_WIN = 2 * FILM_HALO + 1;                      // 9
constexpr int FILM_MASK_WORDS = (FILM_WIN * FILM_WIN + 31) / 32;  // 3
// A sample's footprint spans at most 5 columns and 5 rows (film.rs:90-97); its Mitchell
// factors for the tile columns and rows it covers are evaluated once when it is staged:
// mx[j][k] = mitchell1((cb + j - col_discr) / 2) for tile column cb + j, and my likewise,
// so a pixel's weight is mx * my, the reference's product of the same two factors.
constexpr int FILM_FOOT = 5;
struct StagedSample {
    float r[FILM_SPAN * FILM_SPAN], g[FILM_SPAN * FILM_SPAN], b[FILM_SPAN * FILM_SPAN];
    float mx[FILM_FOOT][FILM_SPAN * FILM_SPAN], my[FILM_FOOT][FILM_SPAN * FILM_SPAN];
    uint8_t cb[FILM_SPAN * FILM_SPAN], rb[FILM_SPAN * FILM_SPAN];  // first covered tile column / row
    uint32_t mask[FILM_TILE * FILM_TILE][FILM_MASK_WORDS];
};

// Adds the samples of `npass` passes, in pass order, to the tile (ox, oy) of `film`.
// src_at(k) gives pass k's sample source: src(row, col, st, rgb) loads that pixel's
// sample, its film position (s, t) and its radiance.  Every thread of the block (256 =
// FILM_TILE^2) must call it; `sm` is the block's staging area.
//
// Per pass: each thread stages up to three samples (film.rs:82-97: continuous position,
// footprint) and sets their bit in the mask of every tile pixel their footprint covers;
// then each pixel adds its contributors, set bits in increasing order, with the Mitchell
// weight of film.rs:100-106.  The footprint is the reference's, clamped to the image
// the same way (film.rs:90-97).
//
// Software-pipelined: the global loads of pass k + 1 are issued into registers before
// pass k is accumulated.  The additions per pixel are the reference's: pass by pass,
// then in increasing sample index.
constexpr int FILM_STAGE_PER_THREAD = (FILM_SPAN * FILM_SPAN + FILM_TILE * FILM_TILE - 1) / (FILM_TILE * FILM_TILE);

template <class SrcAt>
GR_D void gather_passes(StagedSample& sm, uint32_t width, uint32_t height, int ox, int oy, float4& acc,
                        uint32_t npass, const SrcAt& src_at) {
    const int tx = threadIdx.x % FILM_TILE, ty = threadIdx.x / FILM_TILE;
    const int x = ox + tx, y = oy + ty;
    const bool inside = x < static_cast<int>(width) && y < static_cast<int>(height);
    const float wf = static_cast<float>(width), hf = static_cast<float>(height);
    const long long last_col = static_cast<long long>(width) - 1, last_row = static_cast<long long>(height) - 1;
    float2 rs[FILM_STAGE_PER_THREAD];
    V3 rc[FILM_STAGE_PER_THREAD];
    auto load = [&](uint32_t pass) {
        const auto src = src_at(pass);
#pragma unroll
        for (int j = 0; j < FILM_STAGE_PER_THREAD; ++j) {
            int k = threadIdx.x + j * FILM_TILE * FILM_TILE;
            int sr = oy - FILM_HALO + k / FILM_SPAN, sc = ox - FILM_HALO + k % FILM_SPAN;
            if (k < FILM_SPAN * FILM_SPAN && sr >= 0 && sc >= 0 && sr < static_cast<int>(height) &&
                sc < static_cast<int>(width))
                src(static_cast<uint32_t>(sr), static_cast<uint32_t>(sc), rs[j], rc[j]);
        }
    };
    if (npass) load(0);
    for (uint32_t pass = 0; pass < npass; ++pass) {
        __syncthreads();  // the previous pass's accumulation is done with sm
#pragma unroll
        for (int w = 0; w < FILM_MASK_WORDS; ++w) sm.mask[threadIdx.x][w] = 0u;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < FILM_STAGE_PER_THREAD; ++j) {
            int k = threadIdx.x + j * FILM_TILE * FILM_TILE;
            if (k >= FILM_SPAN * FILM_SPAN) break;
            int ky = k / FILM_SPAN, kx = k % FILM_SPAN;
            int sr = oy - FILM_HALO + ky, sc = ox - FILM_HALO + kx;
            if (sr < 0 || sc < 0 || sr >= static_cast<int>(height) || sc >= static_cast<int>(width)) continue;
            float2 s = rs[j];
            // film.rs:82-97
            float col_cont = lerp(0.0f, wf, 0.5f * (s.x + 1.0f));
            float row_cont = lerp(0.0f, hf, 0.5f * (s.y + 1.0f));
            float cd = col_cont - 0.5f, rd = row_cont - 0.5f;
            sm.r[k] = rc[j].x;
            sm.g[k] = rc[j].y;
            sm.b[k] = rc[j].z;
            // Footprint (film.rs:90-97), then the tile pixels it covers; footprints never
            // exceed +-4 px of the source pixel.
            long long mnc = static_cast<long long>(ceilf(cd - 2.0f));
            long long mxc = static_cast<long long>(floorf(cd + 2.0f));
            long long mnr = static_cast<long long>(ceilf(rd - 2.0f));
            long long mxr = static_cast<long long>(floorf(rd + 2.0f));
            mnc = mnc < 0 ? 0 : (mnc > last_col ? last_col : mnc);
            mxc = mxc < 0 ? 0 : (mxc > last_col ? last_col : mxc);
            mnr = mnr < 0 ? 0 : (mnr > last_row ? last_row : mnr);
            mxr = mxr < 0 ? 0 : (mxr > last_row ? last_row : mxr);
            int c0 = max(0, static_cast<int>(mnc) - ox), c1 = min(FILM_TILE - 1, static_cast<int>(mxc) - ox);
            int r0 = max(0, static_cast<int>(mnr) - oy), r1 = min(FILM_TILE - 1, static_cast<int>(mxr) - oy);
            if (c0 > c1 || r0 > r1) continue;  // covers no pixel of this tile
            sm.cb[k] = static_cast<uint8_t>(c0);
            sm.rb[k] = static_cast<uint8_t>(r0);
            // film.rs:100-106 factors, the arguments as the pixel loop below forms them
#pragma unroll
            for (int f = 0; f < FILM_FOOT; ++f)
                if (f <= c1 - c0) sm.mx[f][k] = mitchell1((static_cast<float>(ox + c0 + f) - cd) / 2.0f);
#pragma unroll
            for (int f = 0; f < FILM_FOOT; ++f)
                if (f <= r1 - r0) sm.my[f][k] = mitchell1((static_cast<float>(oy + r0 + f) - rd) / 2.0f);
            for (int py = r0; py <= r1; ++py)
                for (int px = c0; px <= c1; ++px) {
                    int bit = (ky - py) * FILM_WIN + (kx - px);
                    atomicOr(&sm.mask[py * FILM_TILE + px][bit >> 5], 1u << (bit & 31));
                }
        }
        __syncthreads();
        if (pass + 1 < npass) load(pass + 1);  // in flight while this pass accumulates
        if (!inside) continue;
#pragma unroll
        for (int w = 0; w < FILM_MASK_WORDS; ++w) {
            uint32_t m = sm.mask[threadIdx.x][w];
            while (m) {
                int bit = w * 32 + __ffs(m) - 1;
                m &= m - 1;
                int dy = bit / FILM_WIN, dx = bit - dy * FILM_WIN;
                int k = (ty + dy) * FILM_SPAN + (tx + dx);
                float wgt = sm.mx[tx - sm.cb[k]][k] * sm.my[ty - sm.rb[k]][k];
                acc.x = acc.x + sm.r[k] * wgt;
                acc.y = acc.y + sm.g[k] * wgt;
                acc.z = acc.z + sm.b[k] * wgt;
                acc.w += wgt;
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
