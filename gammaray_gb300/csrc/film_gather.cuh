// Deterministic film splat, shared by the per-image render (film.cu) and the engine.
//
// Film::report_samples (render/film.rs:78-114) splats each sample, serially and in
// sample order, over the pixels within 2 px of its jittered position with a Mitchell
// weight.  Samples are jittered less than 2 px from their own pixel centre (the camera
// jitter of film_sample_point), so a sample covers at most 5 consecutive columns and 5
// consecutive rows, all within 4 px of its own pixel.
//
// gather_passes gives each thread one destination pixel of a 24x16 tile.  Per pass, the
// block stages the samples of the tile's 32x24 neighbourhood (the tile and 4 px of halo)
// in shared memory, one warp per neighbourhood row and one lane per column; then every
// pixel adds its contributors in increasing sample index (rows, then columns).  That is
// the order of the reference's serial loop, so the sums are bit-identical to it, with
// no atomics.
#pragma once

#include "common.cuh"
#include "mitchell.cuh"

namespace gr {

constexpr int FILM_TILE_W = 24;
constexpr int FILM_TILE_H = 16;
constexpr int FILM_HALO = 4;
constexpr int FILM_SPAN_W = FILM_TILE_W + 2 * FILM_HALO;  // 32: one lane per neighbourhood column
constexpr int FILM_SPAN_H = FILM_TILE_H + 2 * FILM_HALO;  // 24
constexpr int FILM_SPAN_N = FILM_SPAN_W * FILM_SPAN_H;
constexpr int FILM_THREADS = FILM_TILE_W * FILM_TILE_H;  // 384, one per tile pixel
constexpr int FILM_WARPS = FILM_THREADS / 32;
constexpr int FILM_ROWS_PER_WARP = FILM_SPAN_H / FILM_WARPS;  // 2
constexpr int FILM_WIN = 2 * FILM_HALO + 1;                   // 9 candidate rows and columns per pixel
constexpr int FILM_FOOT = 5;                                  // columns (rows) one sample covers, at most
static_assert(FILM_SPAN_W == 32 && FILM_THREADS % 32 == 0 && FILM_SPAN_H % FILM_WARPS == 0,
              "one warp per neighbourhood row, the rows shared evenly");
// Gather blocks resident per SM, the register cap of the gather kernels (40 registers at
// 4, 56 at 3); 46.8 KB of shared memory per block allows 4.  On the path-tracer workload
// (1024 x 1024, 64 passes) 2 / 3 / 4 measured 4.21 / 3.42 / 3.22 ms of film accumulation.
#ifndef GR_FILM_BLOCKS_PER_SM
#define GR_FILM_BLOCKS_PER_SM 4
#endif

// Film tiles of a width x height image.
GR_HD uint32_t film_tiles_x(uint32_t width) { return (width + FILM_TILE_W - 1) / FILM_TILE_W; }
GR_HD uint32_t film_tiles_y(uint32_t height) { return (height + FILM_TILE_H - 1) / FILM_TILE_H; }

// A tile's staged samples, sample k = row * 32 + column of the neighbourhood:
//   color[k]             its radiance (w unused)
//   mx[t % 5][k]         mitchell1((ox + t - col_discr) / 2) for each tile column t it
//                        covers; its at most 5 consecutive columns have distinct t % 5
//   my[t % 5][k]         likewise for the tile rows t it covers
//   colmask[row][t]      bit c set when sample (row, c) covers tile column t
//   rowmask[row][t]      bit c set when sample (row, c) covers tile row t
// so sample (row, c) covers pixel (tx, ty) when bit c is set in
// colmask[row][tx] & rowmask[row][ty], and its weight there is mx[tx % 5] * my[ty % 5]:
// the reference's product of the same two factors.
struct StagedSample {
    float4 color[FILM_SPAN_N];
    float mx[FILM_FOOT][FILM_SPAN_N], my[FILM_FOOT][FILM_SPAN_N];
    uint32_t colmask[FILM_SPAN_H][FILM_TILE_W], rowmask[FILM_SPAN_H][FILM_TILE_H];
};

// Transposes the 32x32 bit matrix whose row i (bit j = column j) lane i holds: returns
// column `lane` (bit i = row i's bit `lane`).  Recursive block swap: at stride s the
// two s x s blocks off the diagonal of every 2s x 2s block trade places between lanes
// s apart, then the blocks are transposed at stride s / 2.
GR_D uint32_t transpose32(uint32_t x, unsigned lane) {
    const uint32_t m[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const int s = 16 >> i;
        uint32_t y = __shfl_xor_sync(0xffffffffu, x, s);
        x = (lane & s) ? ((x & ~m[i]) | ((y >> s) & m[i])) : ((x & m[i]) | ((y & m[i]) << s));
    }
    return x;
}

// Adds the samples of `npass` passes, in pass order, to the tile (ox, oy) of `film`.
// src_at(k) gives pass k's sample source: src(row, col, st, rgb) loads that pixel's
// sample, its film position (s, t) and its radiance.  Every thread of the block
// (FILM_THREADS) must call it; `sm` is the block's staging area.
//
// Per pass: each lane stages its column's sample in the warp's neighbourhood rows
// (film.rs:82-97: continuous position, footprint clamped to the image as the reference
// clamps it), evaluates the Mitchell factors of the tile columns and rows the footprint
// covers (film.rs:100-106, the arguments as the reference's pixel loop forms them), and
// the warp transposes its lanes' coverage bits into the row's column and row masks.
// Then each pixel adds its contributors, rows then columns in increasing order, which
// is increasing sample index.
//
// Software-pipelined: the global loads of pass k + 1 are issued into registers before
// pass k is accumulated.  The additions per pixel are the reference's: pass by pass,
// then in increasing sample index.
template <class SrcAt>
GR_D void gather_passes(StagedSample& sm, uint32_t width, uint32_t height, int ox, int oy, float4& acc,
                        uint32_t npass, const SrcAt& src_at) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const int tx = static_cast<int>(threadIdx.x) % FILM_TILE_W, ty = static_cast<int>(threadIdx.x) / FILM_TILE_W;
    const bool inside = ox + tx < static_cast<int>(width) && oy + ty < static_cast<int>(height);
    const float wf = static_cast<float>(width), hf = static_cast<float>(height);
    const int last_col = static_cast<int>(width) - 1, last_row = static_cast<int>(height) - 1;
    const int scol = ox - FILM_HALO + static_cast<int>(lane);  // this lane's image column
    const bool col_in = scol >= 0 && scol < static_cast<int>(width);
    const float* mxs = sm.mx[tx % FILM_FOOT];
    const float* mys = sm.my[ty % FILM_FOOT];
    float2 rs[FILM_ROWS_PER_WARP];
    V3 rc[FILM_ROWS_PER_WARP];
    auto load = [&](uint32_t pass) {
        const auto src = src_at(pass);
#pragma unroll
        for (int j = 0; j < FILM_ROWS_PER_WARP; ++j) {
            int srow = oy - FILM_HALO + static_cast<int>(warp) + j * FILM_WARPS;
            if (col_in && srow >= 0 && srow < static_cast<int>(height))
                src(static_cast<uint32_t>(srow), static_cast<uint32_t>(scol), rs[j], rc[j]);
        }
    };
    if (npass) load(0);
    for (uint32_t pass = 0; pass < npass; ++pass) {
        __syncthreads();  // the previous pass's accumulation is done with sm
#pragma unroll
        for (int j = 0; j < FILM_ROWS_PER_WARP; ++j) {
            const int row = static_cast<int>(warp) + j * FILM_WARPS;
            const int srow = oy - FILM_HALO + row;
            const int k = row * FILM_SPAN_W + static_cast<int>(lane);
            uint32_t cm = 0u, rm = 0u;  // tile columns / rows this sample covers
            if (col_in && srow >= 0 && srow < static_cast<int>(height)) {
                float2 s = rs[j];
                // film.rs:82-97
                float col_cont = lerp(0.0f, wf, 0.5f * (s.x + 1.0f));
                float row_cont = lerp(0.0f, hf, 0.5f * (s.y + 1.0f));
                float cd = col_cont - 0.5f, rd = row_cont - 0.5f;
                // The reference converts to i64 (saturating, NaN -> 0) and clamps to the
                // image; a saturating i32 conversion (NaN -> 0 too) clamps the same.
                int mnc = __float2int_rz(ceilf(cd - 2.0f)), mxc = __float2int_rz(floorf(cd + 2.0f));
                int mnr = __float2int_rz(ceilf(rd - 2.0f)), mxr = __float2int_rz(floorf(rd + 2.0f));
                mnc = min(max(mnc, 0), last_col);
                mxc = min(max(mxc, 0), last_col);
                mnr = min(max(mnr, 0), last_row);
                mxr = min(max(mxr, 0), last_row);
                int c0 = max(0, mnc - ox), c1 = min(FILM_TILE_W - 1, mxc - ox);
                int r0 = max(0, mnr - oy), r1 = min(FILM_TILE_H - 1, mxr - oy);
                if (c0 <= c1 && r0 <= r1) {
                    sm.color[k] = make_float4(rc[j].x, rc[j].y, rc[j].z, 0.0f);
#pragma unroll
                    for (int f = 0; f < FILM_FOOT; ++f) {
                        int t = c0 + f;
                        if (t <= c1) sm.mx[t % FILM_FOOT][k] = mitchell1((static_cast<float>(ox + t) - cd) / 2.0f);
                    }
#pragma unroll
                    for (int f = 0; f < FILM_FOOT; ++f) {
                        int t = r0 + f;
                        if (t <= r1) sm.my[t % FILM_FOOT][k] = mitchell1((static_cast<float>(oy + t) - rd) / 2.0f);
                    }
                    cm = (2u << c1) - (1u << c0);
                    rm = (2u << r1) - (1u << r0);
                }
            }
            const uint32_t xc = transpose32(cm, lane), yc = transpose32(rm, lane);
            if (lane < static_cast<unsigned>(FILM_TILE_W)) sm.colmask[row][lane] = xc;
            if (lane < static_cast<unsigned>(FILM_TILE_H)) sm.rowmask[row][lane] = yc;
        }
        __syncthreads();
        if (pass + 1 < npass) load(pass + 1);  // in flight while this pass accumulates
        if (!inside) continue;
#pragma unroll
        for (int dy = 0; dy < FILM_WIN; ++dy) {
            const int row = ty + dy;
            // candidates: columns tx .. tx + 8 of the row (footprints reach 4 px)
            uint32_t m = ((sm.colmask[row][tx] & sm.rowmask[row][ty]) >> tx) & ((1u << FILM_WIN) - 1u);
            while (m) {
                const int k = row * FILM_SPAN_W + tx + __ffs(m) - 1;
                m &= m - 1;
                const float4 c = sm.color[k];
                const float wgt = mxs[k] * mys[k];
                acc.x = acc.x + c.x * wgt;
                acc.y = acc.y + c.y * wgt;
                acc.z = acc.z + c.z * wgt;
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
