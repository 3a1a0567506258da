"""Serving loop: renders admitted by free device memory, their passes interleaved on one
resident multi-job wavefront (gr_server_*).  Scenes stay resident; each request owns a
film on the device until it is taken."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi

STATE_NAMES = {0: "queued", 1: "running", 2: "done", 3: "cancelled", 4: "failed"}


class Server:
    def __init__(self, lib, memory_budget_bytes: int = 0, max_active: int = 0, path_capacity: int = 0,
                 bvh_width: int = 0, block_size: int = 0, policy: int = _abi.SERVE_ARRIVAL_ORDER):
        """policy: _abi.SERVE_ARRIVAL_ORDER (the oldest request first, later ones fill the
        paths it leaves free) or _abi.SERVE_SHORTEST_FIRST (fewest samples left, aged)."""
        self.lib = lib
        o = _abi.ServerOptions(memory_budget_bytes, max_active, path_capacity, bvh_width, block_size, policy)
        h = C.c_void_p()
        lib.call("gr_server_create", C.byref(o), C.byref(h))
        self.handle = h
        self.sizes = {}

    def close(self):
        if self.handle:
            self.lib.gr_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, stage, camera, integrator, width: int, height: int, spp: int, first_pass: int = 0,
               target_rel_mse: float = 0.0) -> int:
        """Queues a render of `spp` passes; with target_rel_mse > 0, passes stop once the
        estimated relative MSE reaches it (spp is then the most passes)."""
        r = _abi.Request()
        r.scene = stage.handle.value
        r.camera = camera.desc()
        r.params = stage.params(integrator, spp, first_pass)
        r.width, r.height = width, height
        r.target_rel_mse = float(target_rel_mse)
        rid = C.c_uint64()
        self.lib.call("gr_server_submit", self.handle, C.byref(r), C.byref(rid))
        self.sizes[rid.value] = (width, height)
        return rid.value

    def step(self, budget_ms: float = 5.0):
        self.lib.call("gr_server_step", self.handle, C.c_double(budget_ms))

    def poll(self, rid: int) -> _abi.RequestStatus:
        s = _abi.RequestStatus()
        self.lib.call("gr_server_poll", self.handle, rid, C.byref(s))
        return s

    def cancel(self, rid: int):
        self.lib.call("gr_server_cancel", self.handle, rid)

    def take(self, rid: int):
        w, h = self.sizes.pop(rid)
        acc = np.empty((h, w, 3), np.float32)
        wt = np.empty((h, w), np.float32)
        self.lib.call("gr_server_take", self.handle, rid, _abi.fptr(acc), _abi.fptr(wt))
        return acc, wt

    def snapshot(self, rid: int):
        """gr_server_snapshot: the request's film so far, (accum, weight, passes)."""
        w, h = self.sizes[rid]
        acc = np.empty((h, w, 3), np.float32)
        wt = np.empty((h, w), np.float32)
        passes = C.c_uint32()
        self.lib.call("gr_server_snapshot", self.handle, rid, _abi.fptr(acc), _abi.fptr(wt), C.byref(passes))
        return acc, wt, passes.value

    def info(self) -> _abi.ServerInfo:
        """gr_server_get_info: requests by state, the engine's table sizes and resets."""
        i = _abi.ServerInfo()
        self.lib.call("gr_server_get_info", self.handle, C.byref(i))
        return i

    def run_until_done(self, ids, budget_ms: float = 20.0, max_steps: int = 3000):
        pending = set(ids)
        for _ in range(max_steps):
            if not pending:
                return
            self.step(budget_ms)
            for rid in list(pending):
                if self.poll(rid).state in (2, 3, 4):
                    pending.discard(rid)
        raise TimeoutError(f"{len(pending)} requests did not finish")
