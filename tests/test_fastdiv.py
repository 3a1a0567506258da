"""Division by a launch-invariant divisor (csrc/common.cuh FastDiv, used for the path
tracer's pixel index arithmetic), compiled for the host from the same source and checked
against integer division."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from gammaray_gb300 import build

PROGRAM = r"""
#include "common.cuh"
#include <cstdio>
#include <random>

int main() {
    std::mt19937 rng(7);
    std::uniform_int_distribution<uint32_t> any(0u, 0xFFFFFFFFu), div31(1u, 0x7FFFFFFFu);
    unsigned long long bad = 0, checks = 0;
    auto check = [&](uint32_t d) {
        const gr::FastDiv f = gr::make_fastdiv(d);
        const uint32_t edge[] = {0u, 1u, d - 1u, d, d + 1u, 2u * d - 1u, 0xFFFFFFFEu, 0xFFFFFFFFu};
        for (uint32_t n : edge) {
            ++checks;
            if (gr::fast_div(n, f) != n / d) ++bad;
        }
        for (int k = 0; k < 64; ++k) {
            const uint32_t n = any(rng);
            ++checks;
            if (gr::fast_div(n, f) != n / d) ++bad;
        }
    };
    for (uint32_t d = 1; d <= 4096; ++d) check(d);
    for (uint32_t d : {576u, 1024u, 1048576u, 2073600u, 3686400u, 0x40000000u, 0x7FFFFFFFu}) check(d);
    for (int k = 0; k < 20000; ++k) check(div31(rng));
    std::printf("%llu %llu\n", checks, bad);
    return bad ? 1 : 0;
}
"""


def test_fast_div_equals_integer_division(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no host C++ compiler")
    here = os.path.dirname(os.path.abspath(build.__file__))
    src = tmp_path / "fastdiv.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "fastdiv"
    cmd = [gxx, "-O2", "-std=c++17", "-I" + os.path.join(build._cuda_home(), "include"),
           "-I" + os.path.join(here, "csrc"), "-I" + os.path.join(here, "..", "include"), str(src), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    checks, bad = (int(x) for x in out.stdout.split())
    assert checks > 1_000_000 and bad == 0 and out.returncode == 0
