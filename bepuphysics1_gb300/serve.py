"""Serving over the C ABI (bepugpu_server_* / bepugpu_serve_*).

A `Server` owns the residency and the steps of the scenes added to it: step
requests are submitted from any thread, run in continuously batched waves on
the device, and come back as completions with their submit, launch and
completion times.  Scenes are given back with `release` (resident, steppable
and downloadable through their GpuSpace again).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native as N
from .solver import Context, GpuSpace


def default_config() -> np.ndarray:
    c = np.zeros(1, N.SERVER_CONFIG_DTYPE)
    N.load_gpu_library().bepugpu_server_default_config(N.ptr(c))
    return c[0].copy()


def clock_us() -> float:
    return N.load_gpu_library().bepugpu_clock_us()


class Server:
    def __init__(self, ctx: Context, budget_bytes: int | None = None, batching: bool = True,
                 max_wave_scenes: int | None = None, waves_in_flight: int | None = None,
                 queue_capacity: int | None = None, dt: float | None = None, flags: int = N.STEP_ALL,
                 threads: int = 0):
        self.ctx = ctx
        self.lib = ctx.lib
        cfg = default_config()
        if budget_bytes is not None:
            cfg["device_budget_bytes"] = int(budget_bytes)
        if max_wave_scenes is not None:
            cfg["max_wave_scenes"] = int(max_wave_scenes)
        if waves_in_flight is not None:
            cfg["max_waves_in_flight"] = int(waves_in_flight)
        if queue_capacity is not None:
            cfg["queue_capacity"] = int(queue_capacity)
        if dt is not None:
            cfg["dt"] = float(dt)
        cfg["batching"] = 1 if batching else 0
        cfg["flags"] = flags
        cfg["threads"] = int(threads)
        self.config = cfg
        h = ctypes.c_void_p()
        c = np.array(cfg, N.SERVER_CONFIG_DTYPE).reshape(1)
        ctx.check(self.lib.bepugpu_server_create(ctx.handle, N.ptr(c), ctypes.byref(h)))
        self.handle = h
        self._buf = np.zeros(4096, N.COMPLETION_DTYPE)

    def check(self, status: int):
        if status != N.OK:
            msg = self.lib.bepugpu_server_last_error(self.handle)
            N.raise_for(status, msg.decode() if msg else "")

    def last_error(self) -> str:
        msg = self.lib.bepugpu_server_last_error(self.handle)
        return msg.decode() if msg else ""

    def add(self, space: GpuSpace):
        self.check(self.lib.bepugpu_server_add_scene(self.handle, space.id))

    def release(self, space: GpuSpace, timeout_ms: int = 60000):
        self.check(self.lib.bepugpu_server_release_scene(self.handle, space.id, timeout_ms))

    def submit(self, scene_id: int, steps: int, tag: int = 0) -> int:
        """Returns the status (OK or QUEUE_FULL) without raising on a full ring."""
        return self.lib.bepugpu_serve_submit(self.handle, int(scene_id), int(steps), int(tag))

    def poll(self) -> np.ndarray:
        n = ctypes.c_uint32()
        self.check(self.lib.bepugpu_serve_poll(self.handle, N.ptr(self._buf), len(self._buf), ctypes.byref(n)))
        return self._buf[:n.value].copy()

    def drain(self, timeout_ms: int = 600000):
        self.check(self.lib.bepugpu_server_drain(self.handle, timeout_ms))

    def stats(self) -> np.void:
        out = np.zeros(1, N.SERVER_STATS_DTYPE)
        self.check(self.lib.bepugpu_server_stats_get(self.handle, N.ptr(out)))
        return out[0]

    def close(self):
        if getattr(self, "handle", None):
            st = self.lib.bepugpu_server_destroy(self.handle)
            self.handle = None
            N.raise_for(st, "bepugpu_server_destroy")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
