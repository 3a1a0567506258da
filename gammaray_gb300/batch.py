"""Batched rendering: many scenes, cameras and films in one multi-job wavefront.

`render_batch(jobs)` calls gr_render_batch: every path-tracer job shares one pool of
path slots, refilled as paths finish, under a captured CUDA graph.  The autotuner picks
all three of its settings by timing short trials:
  - `choose_bvh_width` the BVH width: the scenes are built at widths 2, 4 and 8 (a
    scene's wide BVH is fixed when it is built, so this needs the prims);
  - `autotune(jobs)` the pool capacity and the extension block size (gr_batch_autotune);
  - `autotune_workloads` both in turn, returning the width and the options.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

from . import _abi
from .api import Camera, Film, Stage


@dataclass
class Job:
    stage: Stage
    camera: Camera
    integrator: object
    film: Film
    spp: int

    def desc(self) -> _abi.Job:
        j = _abi.Job()
        j.scene = self.stage.handle.value if isinstance(self.stage.handle, C.c_void_p) else self.stage.handle
        j.camera = self.camera.desc()
        p = self.stage.params(self.integrator, self.spp, first_pass=self.film.passes())
        j.params = p
        j.film = self.film.handle.value if isinstance(self.film.handle, C.c_void_p) else self.film.handle
        return j


def _descs(jobs):
    arr = (_abi.Job * max(1, len(jobs)))(*[j.desc() for j in jobs])
    return arr


def render_batch(jobs, lib, path_capacity: int = 0, block_size: int = 0) -> _abi.RenderStats:
    arr = _descs(jobs)
    opt = _abi.BatchOptions(path_capacity, block_size, 1, 0)
    lib.call("gr_render_batch", arr, len(jobs), C.byref(opt))
    st = _abi.RenderStats()
    lib.call("gr_batch_last_stats", C.byref(st))
    return st


def release(lib):
    """gr_batch_release: frees the engines kept for reuse between batches."""
    lib.call("gr_batch_release")


def autotune(jobs, lib) -> _abi.BatchOptions:
    arr = _descs(jobs)
    opt = _abi.BatchOptions()
    lib.call("gr_batch_autotune", arr, len(jobs), C.byref(opt))
    return opt


def render_individually(jobs, lib) -> float:
    """The plain per-image path on the same requests: one gr_render per job.  Returns
    the summed CUDA-event time in ms."""
    import ctypes as C

    total = 0.0
    for j in jobs:
        p = j.stage.params(j.integrator, j.spp, first_pass=j.film.passes())
        cam = j.camera.desc()
        lib.call("gr_render", j.stage.handle, C.byref(cam), C.byref(p), j.film.handle)
        total += j.stage.last_stats().device_ms
    return total


def render_per_pass(jobs, lib) -> float:
    """The drop-in path: one Stage::trace call (gr_render with spp = 1) per pass."""
    import ctypes as C

    total = 0.0
    for j in jobs:
        cam = j.camera.desc()
        for k in range(j.spp):
            p = j.stage.params(j.integrator, 1, first_pass=j.film.passes())
            lib.call("gr_render", j.stage.handle, C.byref(cam), C.byref(p), j.film.handle)
            total += j.stage.last_stats().device_ms
    return total


def autotune_workloads(workloads, lib, widths=(2, 4, 8), seeds=None):
    """The width trial, then gr_batch_autotune on the scenes built at the chosen width.
    Returns (width, {width: trial Msamples/s}, options, stages at that width)."""
    width, rates = choose_bvh_width(workloads, lib, widths)
    stages = [Stage(w.prims, lib=lib, environment=w.environment, bvh_width=width,
                    seed=(seeds[k] if seeds is not None else 0)) for k, w in enumerate(workloads)]
    jobs = [Job(st, w.camera, w.integrator, Film(w.width, w.height, lib=lib), w.spp)
            for st, w in zip(stages, workloads)]
    opt = autotune(jobs, lib)
    for j in jobs:
        j.film.close()
    return width, rates, opt, stages


def choose_bvh_width(workloads, lib, widths=(2, 4, 8), trial_spp: int = 2):
    """Builds the scenes at each width, renders a short trial batch and returns
    (best width, {width: Msamples/s})."""
    rates = {}
    for wdt in widths:
        jobs = []
        for w in workloads:
            st = Stage(w.prims, lib=lib, environment=w.environment, bvh_width=wdt)
            jobs.append(Job(st, w.camera, w.integrator, Film(w.width, w.height, lib=lib), min(trial_spp, w.spp)))
        t0 = time.perf_counter()
        s = render_batch(jobs, lib)
        dt = s.device_ms if s.device_ms > 0 else (time.perf_counter() - t0) * 1e3
        rates[wdt] = s.samples / dt / 1e3
        for j in jobs:
            j.stage.close()
            j.film.close()
    return max(rates, key=rates.get), rates
