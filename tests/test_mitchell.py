"""The film gather's Mitchell filter (csrc/mitchell.cuh: one cubic with the branch's
coefficients) against the reference's two-branch formula (core/math.rs:92-123), bit for
bit, compiled for the host from the same source without contraction."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from gammaray_gb300 import build

PROGRAM = r"""
#include "mitchell.cuh"
#include <cmath>
#include <cstdio>
#include <cstring>

// core/math.rs:92-123 restated: two branches, sums left to right.
static float reference(float x) {
    const float B = 1.0f / 3.0f, C = 1.0f / 3.0f;
    float twox = std::fabs(2.0f * x);
    if (twox > 1.0f)
        return ((-B - 6.0f * C) * (twox * twox * twox) + (6.0f * B + 30.0f * C) * (twox * twox) +
                (-12.0f * B - 48.0f * C) * twox + (8.0f * B + 24.0f * C)) * (1.0f / 6.0f);
    return ((12.0f - 9.0f * B - 6.0f * C) * (twox * twox * twox) + (-18.0f + 12.0f * B + 6.0f * C) * (twox * twox) +
            (6.0f - 2.0f * B)) * (1.0f / 6.0f);
}

static unsigned long long bad = 0, checks = 0;
static void check(uint32_t bits) {
    float x;
    std::memcpy(&x, &bits, 4);
    const float a = gr::mitchell1(x), b = reference(x);
    uint32_t ab, bb;
    std::memcpy(&ab, &a, 4);
    std::memcpy(&bb, &b, 4);
    ++checks;
    if (ab != bb && !(std::isnan(a) && std::isnan(b))) ++bad;
}

int main() {
    float lo = 0.25f, hi = 2.5f, top = 8.0f;
    uint32_t blo, bhi, btop;
    std::memcpy(&blo, &lo, 4);
    std::memcpy(&bhi, &hi, 4);
    std::memcpy(&btop, &top, 4);
    for (uint32_t s = 0; s < 2; ++s) {
        const uint32_t sign = s ? 0x80000000u : 0u;
        for (uint32_t u = blo; u < bhi; ++u) check(sign | u);            // both branch points
        for (uint32_t u = 0; u < btop; u += 61) check(sign | u);         // the rest below 8
        for (uint32_t u : {0u, 1u, 0x7F800000u, 0x7FC00000u}) check(sign | u);  // 0, denormal, inf, nan
    }
    std::printf("%llu %llu\n", checks, bad);
    return bad ? 1 : 0;
}
"""


def test_mitchell_equals_reference_branches(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no host C++ compiler")
    here = os.path.dirname(os.path.abspath(build.__file__))
    src = tmp_path / "mitchell.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "mitchell"
    cmd = [gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
           "-I" + os.path.join(build._cuda_home(), "include"), "-I" + os.path.join(here, "csrc"),
           "-I" + os.path.join(here, "..", "include"), str(src), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    checks, bad = (int(x) for x in out.stdout.split())
    assert checks > 50_000_000 and bad == 0 and out.returncode == 0
