"""In-tree build of libgammaray_gpu.so for sm_103a.

Every translation unit under csrc/ is compiled in parallel (nvcc for .cu, g++ for
.cpp) into csrc/_build/, then linked into gammaray_gb300/libgammaray_gpu.so with a
static CUDA runtime.  Device code uses -fmad=false and host code -ffp-contract=off so
a*b+c is never fused, matching the reference's Rust arithmetic.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(CSRC, "_build")
LIB = os.path.join(HERE, "libgammaray_gpu.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT_DIR, exist_ok=True)
    inc = ["-I" + os.path.join(HERE, "..", "include"), "-I" + CSRC]
    cu_flags = [nvcc, "-c", "-O3", "-std=c++17", ARCH, "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
                "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", *inc]
    if ptxas_verbose:
        cu_flags += ["-Xptxas", "-v"]
    cu_flags += os.environ.get("GR_NVCC_FLAGS", "").split()
    # -O3 (no fast-math: IEEE arithmetic, the same trees) builds the bench scene's BVH in
    # about 6 ms on 16 Grace cores against 9 ms at -O2.
    cpp_flags = ["g++", "-c", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                 "-I" + os.path.join(cuda, "include"), *inc]
    jobs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        cmd = (cu_flags if src.endswith(".cu") else cpp_flags) + [src, "-o", obj]
        jobs.append((src, obj, cmd))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for src, out in zip(jobs, ex.map(lambda j: _run(j[2]), jobs)):
            logs.append(f"== {os.path.basename(src[0])}\n{out}")
    link = [nvcc, "-shared", ARCH, "-cudart", "static", "-o", LIB] + [j[1] for j in jobs]
    logs.append(_run(link))
    if verbose:
        print("\n".join(logs))
    return "\n".join(logs)


if __name__ == "__main__":
    print(build(verbose=False, ptxas_verbose="-v" in sys.argv))
