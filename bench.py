"""Benchmark: plain per-image GPU path tracing on the 102,400-triangle displaced sphere.

Workload (the configuration the headline metric is quoted on): 1024 x 1024, 64 spp,
max depth 12, FP32; a 160 x 320 UV sphere radially displaced by 3-octave value noise
on a 20-triangle ground plane, one quad light and a constant environment of 0.2, with
per-object Disney parameters from a seed (gammaray_gb300.scenes.displaced_sphere).
One step = one complete render (64 passes of Stage::trace).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Output: one JSON line (rank 0).  `value` is Msamples/s from CUDA events on the render
stream with the scene resident; `e2e` is the same metric through the C ABI with host
buffers (scene build + upload, render, film read-back).  `--impl reference` times the
reference's CPU algorithm (the C++ restatement under oracle/, the reference itself is
Rust and cannot be built here) on all host threads.
Multi-GPU: replicas only (each rank renders its own copy; no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
# DRAM bytes (read + written) per extension ray of k_extend_refill: ncu's
# dram__bytes_read.sum + dram__bytes_write.sum summed over every k_extend_refill launch of
# a 4-spp render of this workload (bench.py --profile-case --spp 4; its 4 M-ray queues
# exceed L2 as the timed renders' do), divided by that render's extension rays.  Re-measured whenever the
# extension kernel changes; EXTEND_DRAM_CAPTURE says which capture the figure comes from.
EXTEND_DRAM_BYTES_PER_RAY = 46.5
EXTEND_DRAM_CAPTURE = "ncu, 4-spp render of the bench workload, all 12 k_extend_refill launches"
sys.path.insert(0, ROOT)

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=1024)
    ap.add_argument("--height", type=int, default=1024)
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    ap.add_argument("--bvh-width", type=int, default=0, help="device BVH width (2, 4, 8); 0 = library default")
    ap.add_argument("--leaf-size", type=int, default=0, help="primitives per wide leaf; 0 = library default")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-rendering measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-bdpt", action="store_true", help="skip the BDPT measurement")
    ap.add_argument("--serve-requests", type=int, default=24)
    ap.add_argument("--serve-rate", type=float, default=3.0, help="Poisson arrival rate (requests/s)")
    ap.add_argument("--serve-target", type=float, default=1e-3,
                    help="relMSE target of the progressive serving leg (0: skip it)")
    ap.add_argument("--profile-bdpt", action="store_true",
                    help="with --profile-case: the BDPT workload (512x512, MIS + light tracing)")
    ap.add_argument("--profile-batch", action="store_true",
                    help="with --profile-case: the 64-scene batch, rendered per image and then in one batch")
    ap.add_argument("--profile-case", action="store_true",
                    help="render the workload once (untimed, --spp passes) and exit: the small case for ncu")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def hbm_peak():
    try:
        with open(MEASURED_PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, n in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(n)
            except Exception:
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def workload(args):
    from gammaray_gb300 import scenes

    return scenes.displaced_sphere(args.width, args.height, args.spp)


def cpu_baseline(w, budget_s, lib=None):
    """The oracle on all host threads over whole 1-spp passes of the same workload until
    the budget is spent (at least one pass)."""
    import gammaray_gb300 as g
    from gammaray_gb300 import _abi

    if lib is None:
        if not os.path.exists(os.path.join(ROOT, "oracle", "libgammaray_ref.so")):
            subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        lib = _abi.Lib(os.path.join(ROOT, "oracle", "libgammaray_ref.so"))
    st = g.Stage(w.prims, lib=lib, environment=w.environment, seed=1)
    film = g.Film(w.width, w.height, lib=lib)
    passes, t0 = 0, time.perf_counter()
    while passes == 0 or time.perf_counter() - t0 < budget_s:
        st.render(w.camera, w.integrator, film, 1)
        passes += 1
    dt = time.perf_counter() - t0
    samples = passes * w.width * w.height
    cores = int(os.environ.get("GR_ORACLE_THREADS", os.cpu_count() or 1))
    return {"value": samples / dt / 1e6, "unit": "Msamples/s", "cores": cores, "kind": "port",
            "sample": f"{passes} x 1-spp pass(es) of the {w.width}x{w.height} workload ({samples} samples, "
                      f"{dt:.1f} s, serial film splat as the reference)"}


def run_reference(args, rank):
    if rank != 0:
        return
    if not os.path.exists(os.path.join(ROOT, "oracle", "libgammaray_ref.so")):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    w = workload(args)
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps))
    for _ in range(args.warmup):
        cpu_baseline(w, 0.0)
    vals = [cpu_baseline(w, per_step) for _ in range(args.steps)]
    v = statistics.median(x["value"] for x in vals)
    cb = dict(vals[0])
    cb["value"] = v
    ms = w.width * w.height * w.spp / (v * 1e6) * 1e3
    line = {"impl": "reference", "metric": "Msamples/s", "value": v, "unit": "Msamples/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_of(w), "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_of(w):
    return {"workload": "pt_displaced_sphere_102k", "width": w.width, "height": w.height, "spp": w.spp,
            "max_depth": w.integrator.max_depth, "triangles": w.num_triangles(), "integrator": "path_tracer",
            "bvh": "reference SAH, collapsed to a wide BVH", "l2": "flushed (256 MiB write) between timed steps",
            "unit_of_step": "one complete render"}


def percentiles(xs):
    xs = np.asarray(xs, np.float64)
    return {"p50": float(np.percentile(xs, 50)), "p95": float(np.percentile(xs, 95)),
            "p99": float(np.percentile(xs, 99)), "mean": float(xs.mean())}


def run_batched(lib):
    """Config 4: 64 seeded scenes (1k-200k triangles, 0-8 spheres, random resolution, spp
    4-64, depth 4-12) rendered (a) one gr_render per image and (b) in one batch, with the
    BVH width, path capacity and block size picked by the autotuner.  Then the same
    comparison per resolution class (a batch of that class's images against their
    per-image renders), which shows where the batch gains and where it cannot."""
    import gammaray_gb300 as g
    from gammaray_gb300 import batch, scenes

    ws = scenes.batch_scenes(64)
    width, width_rates, opt, stages = batch.autotune_workloads(ws, lib, seeds=list(range(len(ws))))
    samples = sum(w.width * w.height * w.spp for w in ws)

    def jobs(idx=None):
        idx = range(len(ws)) if idx is None else idx
        return [batch.Job(stages[k], ws[k].camera, ws[k].integrator, g.Film(ws[k].width, ws[k].height, lib=lib),
                          ws[k].spp) for k in idx]

    # plain per-image path (warm once, then timed)
    warm = jobs()
    batch.render_individually(warm[:4], lib)
    pj = jobs()
    t0 = time.perf_counter()
    plain_dev = batch.render_individually(pj, lib)
    plain_wall = time.perf_counter() - t0
    qj = jobs()
    t0 = time.perf_counter()
    batch.render_per_pass(qj, lib)
    per_pass_wall = time.perf_counter() - t0
    batch.render_batch(jobs()[:8], lib, opt.path_capacity, opt.block_size)  # warm
    bj = jobs()
    t0 = time.perf_counter()
    st = batch.render_batch(bj, lib, opt.path_capacity, opt.block_size)
    batch_wall = time.perf_counter() - t0
    # same requests, same films (bit-identical is tested; spot-check one here)
    a = bj[0].film.read()[0]
    b = pj[0].film.read()[0]
    same = bool(np.allclose(a, b, rtol=1e-6, atol=1e-7))
    # Per resolution class, device time: the class's images per image, then as one batch.
    classes = {}
    for res in sorted({(w.width, w.height) for w in ws}):
        idx = [k for k, w in enumerate(ws) if (w.width, w.height) == res]
        n = sum(ws[k].width * ws[k].height * ws[k].spp for k in idx)
        per_image_ms = batch.render_individually(jobs(idx), lib)
        bs = batch.render_batch(jobs(idx), lib, opt.path_capacity, opt.block_size)
        classes[f"{res[0]}x{res[1]}"] = {
            "images": len(idx), "samples": n, "share_of_samples": n / samples,
            "per_image_ms": per_image_ms, "batch_ms": bs.device_ms,
            "per_image_msamples_per_s": n / (per_image_ms * 1e-3) / 1e6,
            "batch_msamples_per_s": n / (bs.device_ms * 1e-3) / 1e6, "speedup": per_image_ms / bs.device_ms}
    # The classes' batched times added up, against their per-image times; and the
    # ceiling of any batching: every sample at the saturated per-image rate (the best
    # class's, where one image fills the GPU), so the batch's time is at least its
    # samples at that rate.
    t_plain = sum(c["per_image_ms"] for c in classes.values())
    t_batched = sum(c["batch_ms"] for c in classes.values())
    sat_class = max(classes, key=lambda k: classes[k]["per_image_msamples_per_s"])
    sat_rate = classes[sat_class]["per_image_msamples_per_s"]
    ceiling = t_plain / (samples / sat_rate * 1e-3)
    return {"workload": "batch_64_scenes", "samples": samples,
            "msamples_per_s": samples / batch_wall / 1e6, "msamples_per_s_device": samples / (st.device_ms * 1e-3) / 1e6,
            "plain_msamples_per_s": samples / plain_wall / 1e6,
            "plain_msamples_per_s_device": samples / (plain_dev * 1e-3) / 1e6,
            "speedup_vs_plain": plain_wall / batch_wall, "speedup_vs_plain_device": plain_dev / st.device_ms,
            "mrays_per_s": st.extension_rays / batch_wall / 1e6,
            "plain_per_pass_msamples_per_s": samples / per_pass_wall / 1e6,
            "speedup_vs_per_pass": per_pass_wall / batch_wall,
            "autotuned": {"bvh_width": width, "width_trial_msamples_per_s": {str(k): v for k, v in width_rates.items()},
                          "path_capacity": opt.path_capacity, "block_size": opt.block_size},
            "per_class": classes, "per_class_speedup_combined": t_plain / t_batched,
            "speedup_ceiling_at_saturated_rate": ceiling,
            "saturated_class": sat_class, "saturated_msamples_per_s": sat_rate, "films_equal_plain": same}


def run_served(lib, n_req, rate, seed=11, target_rel_mse=1e-3, other_policy=True):
    """Config 5: 16 resident scenes (10k-2M triangles); Poisson arrivals; random pose,
    resolution 256^2..1920x1080, spp 1-256, depth 4-16.  Served by the continuous-
    batching loop (arrival order with backfill, the default policy) vs a FIFO timeline of
    one gr_render per request on the same GPU; then the same requests under the
    shortest-remaining-work policy.  Both latencies run from the request's arrival."""
    import gammaray_gb300 as g
    from gammaray_gb300 import _abi, scenes, serve

    rng = np.random.default_rng(seed)
    scs = scenes.serving_scenes(16)
    stages = [g.Stage(p, lib=lib, environment=env, seed=k) for k, (p, env) in enumerate(scs)]
    resolutions = [(256, 256), (512, 512), (640, 480), (1280, 720), (1920, 1080)]
    reqs = []
    t = 0.0
    for k in range(n_req):
        t += float(rng.exponential(1.0 / rate))
        res = resolutions[int(rng.integers(0, len(resolutions)))]
        reqs.append(dict(arrival=t, scene=int(rng.integers(0, 16)), res=res, spp=int(rng.integers(1, 257)),
                         depth=int(rng.integers(4, 17)), cam=scenes.orbit_camera(rng, *res)))
    samples = sum(r["res"][0] * r["res"][1] * r["spp"] for r in reqs)
    # plain: one render per request, FIFO on one GPU
    dur = []
    for r in reqs:
        f = g.Film(*r["res"], lib=lib)
        integ = g.PathTracerIntegrator(max_depth=r["depth"])
        t0 = time.perf_counter()
        stages[r["scene"]].render(r["cam"], integ, f, r["spp"])
        dur.append(time.perf_counter() - t0)
        f.close()
    finish, lat_plain = 0.0, []
    for r, d in zip(reqs, dur):
        start = max(finish, r["arrival"])
        finish = start + d
        lat_plain.append((finish - r["arrival"]) * 1e3)
    plain_span = finish - reqs[0]["arrival"]
    def serve_all(policy):
        srv = serve.Server(lib, max_active=16, policy=policy)
        ids, late = {}, {}
        t0 = time.perf_counter()
        nxt = 0
        while nxt < len(reqs) or any(srv.poll(i).state < 2 for i in ids.values()):
            now = time.perf_counter() - t0
            while nxt < len(reqs) and reqs[nxt]["arrival"] <= now:
                r = reqs[nxt]
                ids[nxt] = srv.submit(stages[r["scene"]], r["cam"], g.PathTracerIntegrator(max_depth=r["depth"]),
                                      r["res"][0], r["res"][1], r["spp"])
                late[nxt] = (time.perf_counter() - t0 - r["arrival"]) * 1e3  # arrival -> submission
                nxt += 1
            if nxt < len(reqs) and not any(srv.poll(i).state < 2 for i in ids.values()):
                time.sleep(max(0.0, reqs[nxt]["arrival"] - now))
                continue
            srv.step(2.0)
        span = time.perf_counter() - t0 - reqs[0]["arrival"]
        lat = []
        for k, rid in ids.items():
            st = srv.poll(rid)
            lat.append(st.finish_ms - st.submit_ms + late[k])  # from the request's arrival
            srv.take(rid)
        srv.close()
        return span, lat

    span, lat = serve_all(_abi.SERVE_ARRIVAL_ORDER)
    out = {"workload": "serve_16_scenes", "requests": n_req, "rate_per_s": rate, "samples": samples,
           "policy": "arrival order with backfill",
           "msamples_per_s": samples / span / 1e6, "latency_ms": percentiles(lat),
           "plain_fifo_msamples_per_s": samples / plain_span / 1e6, "plain_fifo_latency_ms": percentiles(lat_plain),
           "plain_busy_msamples_per_s": samples / sum(dur) / 1e6,
           "speedup_vs_plain_fifo": plain_span / span,
           "requests_slower_than_fifo": int(sum(a > b for a, b in zip(lat, lat_plain))),
           "per_request": {"fields": ["width", "height", "spp", "max_depth", "arrival_ms", "alone_ms", "fifo_ms",
                                      "served_ms"],
                           "rows": [[r["res"][0], r["res"][1], r["spp"], r["depth"], round(r["arrival"] * 1e3, 1),
                                     round(d * 1e3, 1), round(lp, 1), round(ls, 1)]
                                    for r, d, lp, ls in zip(reqs, dur, lat_plain, lat)]}}
    if other_policy:
        span2, lat2 = serve_all(_abi.SERVE_SHORTEST_FIRST)
        out["shortest_first"] = {"msamples_per_s": samples / span2 / 1e6, "latency_ms": percentiles(lat2),
                                 "speedup_vs_plain_fifo": plain_span / span2}
    if target_rel_mse > 0:
        out["progressive"] = run_progressive(lib, g, serve, stages, reqs, target_rel_mse)
    return out


PROGRESSIVE_MAX_PASSES = 4096


def run_progressive(lib, g, serve, stages, reqs, target):
    """The same requests refined progressively: each stops at the first checkpoint whose
    half-film relMSE estimate is <= target (checkpoints after 8 passes, then where the
    last estimate predicts the target), or at 4096 passes (the drawn spp is not used
    here: relMSE, not a pass count, ends a request).  The plain comparator renders each request's final pass count with one
    gr_render, FIFO, as if it had known the count in advance."""
    srv = serve.Server(lib, max_active=16)
    ids, late = {}, {}
    t0 = time.perf_counter()
    nxt = 0
    while nxt < len(reqs) or any(srv.poll(i).state < 2 for i in ids.values()):
        now = time.perf_counter() - t0
        while nxt < len(reqs) and reqs[nxt]["arrival"] <= now:
            r = reqs[nxt]
            ids[nxt] = srv.submit(stages[r["scene"]], r["cam"], g.PathTracerIntegrator(max_depth=r["depth"]),
                                  r["res"][0], r["res"][1], PROGRESSIVE_MAX_PASSES, target_rel_mse=target)
            late[nxt] = (time.perf_counter() - t0 - r["arrival"]) * 1e3
            nxt += 1
        if nxt < len(reqs) and not any(srv.poll(i).state < 2 for i in ids.values()):
            time.sleep(max(0.0, reqs[nxt]["arrival"] - now))
            continue
        srv.step(2.0)
    span = time.perf_counter() - t0 - reqs[0]["arrival"]
    lat, passes, met, est = [], [], 0, []
    for k, rid in ids.items():
        st = srv.poll(rid)
        lat.append(st.finish_ms - st.submit_ms + late[k])  # from the request's arrival
        passes.append(int(st.passes_done))
        est.append(float(st.rel_mse))
        met += st.rel_mse <= target
        srv.take(rid)
    srv.close()
    samples = sum(r["res"][0] * r["res"][1] * n for r, n in zip(reqs, passes))
    finish, lat_plain, busy = 0.0, [], 0.0
    for r, n in zip(reqs, passes):
        f = g.Film(*r["res"], lib=lib)
        t1 = time.perf_counter()
        stages[r["scene"]].render(r["cam"], g.PathTracerIntegrator(max_depth=r["depth"]), f, n)
        d = time.perf_counter() - t1
        f.close()
        busy += d
        start = max(finish, r["arrival"])
        finish = start + d
        lat_plain.append((finish - r["arrival"]) * 1e3)
    plain_span = finish - reqs[0]["arrival"]
    hist = {str(n): passes.count(n) for n in sorted(set(passes))}
    return {"target_rel_mse": target, "reached_target": int(met), "passes_histogram": hist,
            "rel_mse_estimate": percentiles(est), "samples": samples,
            "msamples_per_s": samples / span / 1e6, "latency_ms": percentiles(lat),
            "plain_fifo_msamples_per_s": samples / plain_span / 1e6, "plain_fifo_latency_ms": percentiles(lat_plain),
            "plain_busy_msamples_per_s": samples / busy / 1e6, "speedup_vs_plain_fifo": plain_span / span}


def run_ours(args, rank, world, local):
    import ctypes as C

    import torch

    import gammaray_gb300 as g
    from gammaray_gb300 import _abi

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    lib = g.load()
    w = workload(args)
    st = g.Stage(w.prims, lib=lib, environment=w.environment, seed=1, bvh_width=args.bvh_width,
                 leaf_size=args.leaf_size)
    info = st.info()
    film = g.Film(w.width, w.height, lib=lib)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    samples_per_step = w.width * w.height * w.spp

    def render(flags=0, spp=None, first=None):
        p = st.params(w.integrator, spp or w.spp, first)
        p.flags = flags
        cam = w.camera.desc()
        lib.call("gr_render", st.handle, C.byref(cam), C.byref(p), film.handle)
        return st.last_stats()

    # Traversal counts per extension ray (untimed, one pass).
    cs = render(_abi.RENDER_COUNT_TRAVERSAL, spp=1)
    nodes_per_ray = cs.node_visits / max(1, cs.extension_rays)
    prims_per_ray = cs.prim_tests / max(1, cs.extension_rays)
    for _ in range(args.warmup):
        render()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    dev_ms, ext_ms, ext_launch, rays, launches, shade_ms = [], 0.0, 0, 0, 0, 0.0
    raygen_ms, film_ms = 0.0, 0.0
    barrier()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            s = render(_abi.RENDER_TIME_KERNELS)
            dev_ms.append(s.device_ms)
            ext_ms += s.extend_ms
            shade_ms += s.shade_ms
            raygen_ms += s.raygen_ms
            film_ms += s.film_ms
            ext_launch += s.extend_launches
            rays += s.extension_rays
            launches += s.kernel_launches
        barrier()
        wall = time.perf_counter() - t0
    from gammaray_gb300 import replicas

    total_ms, all_samples = replicas.aggregate(sum(dev_ms), args.steps * samples_per_step)
    _, all_rays = replicas.aggregate(0.0, rays)
    value = all_samples / (total_ms * 1e-3) / 1e6
    mrays = all_rays / (total_ms * 1e-3) / 1e6

    # End to end through the C ABI with host buffers: scene build + upload, render, read-back.
    e2e_ms, h2d, d2h = [], 0, 0
    # The step's result is read into pinned host memory (numpy views of pinned buffers).
    acc = torch.empty((w.height, w.width, 3), dtype=torch.float32, pin_memory=True).numpy()
    wt = torch.empty((w.height, w.width), dtype=torch.float32, pin_memory=True).numpy()
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        st2 = g.Stage(w.prims, lib=lib, environment=w.environment, seed=1)
        f2 = g.Film(w.width, w.height, lib=lib)
        st2.render(w.camera, w.integrator, f2, w.spp)
        lib.call("gr_film_read", f2.handle, _abi.fptr(acc), _abi.fptr(wt))
        e2e_ms.append((time.perf_counter() - t1) * 1e3)
        h2d = st2.info().device_bytes
        d2h = acc.nbytes + wt.nbytes
        st2.close()
        f2.close()
    e2e = {"value": world * samples_per_step / (statistics.median(e2e_ms) * 1e-3) / 1e6, "unit": "Msamples/s",
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
           "includes": "host SAH build + wide collapse + upload, 64-spp render, film read-back into pinned host memory"}

    # The same render on a tree built on the GPU (GR_BUILD_DEVICE_LBVH), and end to end with
    # that build: the reference's host SAH build is the default and the headline.
    dev_build = None
    if rank == 0:
        g.Stage(w.prims[-1:], lib=lib, device_build=True).close()  # build kernels loaded
        std = g.Stage(w.prims, lib=lib, environment=w.environment, seed=1, device_build=True)
        fd = g.Film(w.width, w.height, lib=lib)
        std.render(w.camera, w.integrator, fd, 2)
        dms = []
        for _ in range(max(1, args.steps)):
            fd.clear()
            flush.zero_()
            torch.cuda.synchronize()
            std.render(w.camera, w.integrator, fd, w.spp)
            dms.append(std.last_stats().device_ms)
        dinfo = std.info()
        de2e = []
        for _ in range(max(1, args.steps)):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            st3 = g.Stage(w.prims, lib=lib, environment=w.environment, seed=1, device_build=True)
            f3 = g.Film(w.width, w.height, lib=lib)
            st3.render(w.camera, w.integrator, f3, w.spp)
            lib.call("gr_film_read", f3.handle, _abi.fptr(acc), _abi.fptr(wt))
            de2e.append((time.perf_counter() - t1) * 1e3)
            st3.close()
            f3.close()
        dev_build = {"build_ms_device": dinfo.build_seconds * 1e3, "build_ms_host_sah": info.build_seconds * 1e3,
                     "wide_nodes": int(dinfo.num_wide_nodes),
                     "msamples_per_s": samples_per_step / (statistics.median(dms) * 1e-3) / 1e6,
                     "e2e_msamples_per_s": samples_per_step / (statistics.median(de2e) * 1e-3) / 1e6}
        std.close()
        fd.close()

    # Roofline of the dominant kernel (extension / closest hit): counted bytes per ray.
    # A node is 32W bytes; at widths 4 and 8 the kernel reads its 7 rows of W floats
    # (bounds and children), not the padding row.
    node_bytes = 28 * info.bvh_width if info.bvh_width % 4 == 0 else 32 * info.bvh_width
    b_ray = nodes_per_ray * node_bytes + prims_per_ray * 48 + 48
    achieved = b_ray * rays / (ext_ms * 1e-3) / 1e9 if ext_ms > 0 else None
    peak, peak_kind = hbm_peak()
    roofline = {"bound": "hbm", "kernel": "k_extend_refill (closest-hit traversal)", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": (achieved / peak) if achieved else None, "traffic": None,
                "peak_source": peak_kind,
                "bytes_per_ray": b_ray, "nodes_per_ray": nodes_per_ray, "prims_per_ray": prims_per_ray,
                "extend_share_of_device_time": ext_ms / total_ms if total_ms else None,
                "shade_share_of_device_time": shade_ms / total_ms if total_ms else None,
                "extend_ms_per_launch": ext_ms / max(1, ext_launch)}
    # Where a render's device time goes (CUDA events on the render stream, per render):
    # the rest is queue-length copies, counter resets and launch gaps between kernels.
    per = float(args.steps)
    breakdown = {"extend": ext_ms / per, "shade": shade_ms / per, "raygen": raygen_ms / per, "film": film_ms / per}
    breakdown["between_launches"] = sum(dev_ms) / per - sum(breakdown.values())
    # DRAM traffic of k_extend per launch: the captured bytes per ray (see
    # EXTEND_DRAM_BYTES_PER_RAY) times the rays of an average timed launch.
    roofline["traffic"] = EXTEND_DRAM_BYTES_PER_RAY * rays / max(1, ext_launch)
    roofline["traffic_source"] = (f"{EXTEND_DRAM_CAPTURE}: {EXTEND_DRAM_BYTES_PER_RAY} B/ray, "
                                  "x rays per timed launch")

    batched = served = bdpt = cornell = None
    if rank == 0 and not args.no_bdpt:
        bdpt = run_bdpt(lib, min(args.cpu_seconds, 8.0))
        cornell = run_cornell(lib, min(args.cpu_seconds, 3.0))
    if rank == 0 and not args.no_batch:
        batched = run_batched(lib)
    if rank == 0 and not args.no_serve:
        served = run_served(lib, args.serve_requests, args.serve_rate, target_rel_mse=args.serve_target)
    if rank == 0:
        cb = cpu_baseline(w, args.cpu_seconds) if world == 1 else None
        line = {"metric": "Msamples/s", "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": config_of(w), "mrays_per_s": mrays, "roofline": roofline,
                "device_ms_per_render": breakdown, "cpu_baseline": cb, "e2e": e2e,
                "gpu_launches": int(launches), "clocks": clk.summary(), "wall_s": wall,
                "batched": batched, "served": served, "bdpt": bdpt, "cornell": cornell, "device_build": dev_build,
                "scene": {"components": int(info.num_components), "wide_nodes": int(info.num_wide_nodes),
                          "device_bytes": int(info.device_bytes), "build_s": info.build_seconds}}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_bdpt(lib, cpu_seconds):
    """Config 3: BDPT on the 102,400-triangle scene at 512x512, 16 spp, path length 10,
    with power-heuristic MIS and light-tracing splats (and, beside it, the reference's
    uniform weights).  Device time per render; rays = extension + shadow rays."""
    import gammaray_gb300 as g
    from gammaray_gb300 import _abi, scenes

    w = scenes.displaced_sphere(512, 512, 16, bdpt=True)
    st = g.Stage(w.prims, lib=lib, environment=w.environment, seed=3)
    samples = w.width * w.height * w.spp
    out = {"workload": "bdpt_displaced_sphere_102k", "width": w.width, "height": w.height, "spp": w.spp,
           "max_path_length": 10}
    forms = (("mis_light_tracing", g.BdptIntegrator(max_depth=10, rr_depth=4, mis=1, light_tracing=1)),
             ("reference_weights", g.BdptIntegrator(max_depth=10, rr_depth=4)))
    for name, integ in forms:
        f = g.Film(w.width, w.height, lib=lib)
        st.render(w.camera, integ, f, 2)  # warm
        ms, s = [], None
        for _ in range(3):
            f.clear()
            st.render(w.camera, integ, f, w.spp)
            s = st.last_stats()
            ms.append(s.device_ms)
        t = statistics.median(ms)
        out[name] = {"msamples_per_s": samples / (t * 1e-3) / 1e6,
                     "mrays_per_s": (s.extension_rays + s.shadow_rays) / (t * 1e-3) / 1e6,
                     "extension_rays": int(s.extension_rays), "shadow_rays": int(s.shadow_rays),
                     "device_ms": t}
        f.close()
    # The oracle on the host cores, whole 1-spp passes of the same workload (MIS + light tracing).
    orc = _abi.Lib(os.path.join(ROOT, "oracle", "libgammaray_ref.so"))
    so = g.Stage(w.prims, lib=orc, environment=w.environment, seed=3)
    fo = g.Film(w.width, w.height, lib=orc)
    passes, t0 = 0, time.perf_counter()
    while passes == 0 or time.perf_counter() - t0 < cpu_seconds:
        so.render(w.camera, forms[0][1], fo, 1)
        passes += 1
    dt = time.perf_counter() - t0
    out["cpu_oracle_msamples_per_s"] = passes * w.width * w.height / dt / 1e6
    out["cpu_oracle_sample"] = f"{passes} x 1-spp pass(es), {dt:.1f} s, {os.cpu_count()} threads"
    return out


def run_cornell(lib, cpu_seconds):
    """Config 1: the closed box with two spheres, path tracer, 256x256, 16 spp, max depth 8,
    roulette after depth 3; device time of the GPU render beside the oracle on the host
    cores (whole 1-spp passes of the same workload)."""
    import gammaray_gb300 as g
    from gammaray_gb300 import _abi, scenes

    w = scenes.cornell_spheres(256, 256, 16)
    st = g.Stage(w.prims, lib=lib, seed=7)
    f = g.Film(w.width, w.height, lib=lib)
    st.render(w.camera, w.integrator, f, 2)  # warm
    ms = []
    for _ in range(5):
        f.clear()
        st.render(w.camera, w.integrator, f, w.spp)
        ms.append(st.last_stats().device_ms)
    samples = w.width * w.height * w.spp
    t = statistics.median(ms)
    orc = _abi.Lib(os.path.join(ROOT, "oracle", "libgammaray_ref.so"))
    so = g.Stage(w.prims, lib=orc, seed=7)
    fo = g.Film(w.width, w.height, lib=orc)
    passes, t0 = 0, time.perf_counter()
    while passes == 0 or time.perf_counter() - t0 < cpu_seconds:
        so.render(w.camera, w.integrator, fo, 1)
        passes += 1
    dt = time.perf_counter() - t0
    return {"workload": "pt_cornell_spheres", "width": w.width, "height": w.height, "spp": w.spp, "max_depth": 8,
            "msamples_per_s": samples / (t * 1e-3) / 1e6, "device_ms": t,
            "cpu_oracle_msamples_per_s": passes * w.width * w.height / dt / 1e6,
            "cpu_oracle_sample": f"{passes} x 1-spp pass(es), {dt:.1f} s, {os.cpu_count()} threads"}


def profile_case(args):
    import gammaray_gb300 as g
    from gammaray_gb300 import batch, scenes

    lib = g.load()
    if args.profile_batch:  # the batch line's 64 scenes: per image, then one batch (64 M paths)
        ws = scenes.batch_scenes(64)
        stages = [g.Stage(w.prims, lib=lib, environment=w.environment, seed=k) for k, w in enumerate(ws)]

        def jobs():
            return [batch.Job(st, w.camera, w.integrator, g.Film(w.width, w.height, lib=lib), w.spp)
                    for st, w in zip(stages, ws)]

        dev = batch.render_individually(jobs(), lib)
        st = batch.render_batch(jobs(), lib, 1 << 26, 256)
        print(json.dumps({"profile_case": "batch_64_scenes", "per_image_device_ms": dev, "batch_device_ms": st.device_ms,
                          "samples": int(st.samples), "rays": int(st.extension_rays)}))
        return
    if args.profile_bdpt:  # the BDPT line's scene and integrator (MIS + light tracing)
        w = scenes.displaced_sphere(512, 512, args.spp or 1, bdpt=True)
        w.integrator = g.BdptIntegrator(max_depth=10, rr_depth=4, mis=1, light_tracing=1)
    else:
        w = workload(args)
    st = g.Stage(w.prims, lib=lib, environment=w.environment, seed=1)
    film = g.Film(w.width, w.height, lib=lib)
    st.render(w.camera, w.integrator, film, w.spp)
    s = st.last_stats()
    case = {"workload": "bdpt_displaced_sphere_102k", "width": w.width, "height": w.height, "spp": w.spp} \
        if args.profile_bdpt else config_of(w)
    print(json.dumps({"profile_case": case, "device_ms": s.device_ms, "rays": s.extension_rays,
                      "launches": s.kernel_launches}))


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.profile_case:
        profile_case(args)
    elif args.impl == "reference":
        run_reference(args, rank)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
