// The reference's Mitchell filter (B = C = 1/3), shared by the film gather and its
// host-side test.
#pragma once

#include "common.cuh"

namespace gr {

// core/math.rs:92-123 (B = C = 1/3): for |2x| > 1
//   ((-B - 6C) |2x|^3 + (6B + 30C) |2x|^2 + (-12B - 48C) |2x| + (8B + 24C)) / 6,
// else ((12 - 9B - 6C) |2x|^3 + (-18 + 12B + 6C) |2x|^2 + (6 - 2B)) / 6, each sum taken
// left to right.  One polynomial with the branch's coefficients: the inner branch's
// missing linear term is + 0 * |2x|, which leaves its partial sum (never -0) unchanged,
// so the result is bit-identical to evaluating the branches without computing both
// (tests/test_mitchell.py: every float with 0.25 <= |x| < 2.5, around both branch
// points, and a stride of the rest below 8).
GR_HD float mitchell1(float x) {
    const float B = 1.0f / 3.0f;
    const float C = 1.0f / 3.0f;
    const float twox = fabsf(2.0f * x);
    const bool outer = twox > 1.0f;
    const float a3 = outer ? (-B - 6.0f * C) : (12.0f - 9.0f * B - 6.0f * C);
    const float a2 = outer ? (6.0f * B + 30.0f * C) : (-18.0f + 12.0f * B + 6.0f * C);
    const float a1 = outer ? (-12.0f * B - 48.0f * C) : 0.0f;
    const float a0 = outer ? (8.0f * B + 24.0f * C) : (6.0f - 2.0f * B);
    const float t2 = twox * twox, t3 = t2 * twox;
    return (((a3 * t3) + (a2 * t2)) + (a1 * twox) + a0) * (1.0f / 6.0f);
}

}  // namespace gr
