"""The serving loop (``pbrtgpu_server_*``): resident scenes, render and
ray-query requests from any thread, continuous batching on the device.

The native worker thread packs waiting requests, oldest first, into the
first free batch slot (as many as its device-memory limits hold) and
launches it at once; up to ``slots`` batches run together.  Each result is
the one the single-request call (``GpuSamplerRenderer.render``,
``GpuBVHAccel.intersect`` / ``intersect_p``) gives, alone or in any mix.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .batch import _KERNEL, limits as batch_limits
from .gpu import GpuBVHAccel, GpuSamplerRenderer, GpuScene, _is_torch, _ray_buffer, _torch


class GpuServer:
    """pool_bytes > 0 holds resident scenes (``admit``) and the slots' arenas
    to that device-memory budget; requests must then name resident scenes
    or BVHs."""

    def __init__(self, slots: int = 2, tuning: dict | None = None, pool_bytes: int = 0, **limit_kw):
        self._lib = abi.load()
        self._resident = []
        cfg = abi.PbrtServerConfig()
        cfg.slots = slots
        cfg.limits = batch_limits(**limit_kw)
        cfg.pool_bytes = int(pool_bytes)
        if tuning:
            cfg.use_tuning = 1
            t = abi.PbrtBatchTuning()
            base = dict(extend_kernel="wide", shadow_kernel="wide", block=128, stack=16, chunk=64, refill=32,
                        refill_shadow=8, use_graph=1)
            base.update(tuning)
            for k, v in base.items():
                setattr(t, k, _KERNEL[v] if k in ("extend_kernel", "shadow_kernel") else int(v))
            cfg.tuning = t
        self.config = cfg
        h = C.c_void_p()
        abi.check(self._lib.pbrtgpu_server_create(C.byref(cfg), C.byref(h)), self._lib)
        self._h = h
        self._keep = {}  # ticket -> buffers the request uses, and its output

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.pbrtgpu_server_destroy(self._h)
        self._h = None
        self._keep = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def admit(self, item) -> None:
        """Makes a GpuScene (with its BVH) or a GpuBVHAccel resident in the
        pool; raises PbrtError(PBRT_ERR_BUDGET) when it does not fit."""
        sc, bvh = (item._h, None) if isinstance(item, GpuScene) else (None, item._h)
        abi.check(self._lib.pbrtgpu_server_admit(self._h, sc, bvh), self._lib)
        self._resident.append(item)  # handles stay alive while resident

    def release(self, item) -> None:
        sc, bvh = (item._h, None) if isinstance(item, GpuScene) else (None, item._h)
        abi.check(self._lib.pbrtgpu_server_release(self._h, sc, bvh), self._lib)
        self._resident = [x for x in self._resident if x is not item]

    def submit_render(self, scene: GpuScene, renderer: GpuSamplerRenderer, out=None) -> int:
        x0, x1, y0, y1 = renderer.pixel_extent()
        if out is None:
            out = np.zeros((y1 - y0, x1 - x0, 3), dtype=np.float32)
        ptr = C.c_void_p(out.data_ptr() if _is_torch(out) else out.ctypes.data)
        t = C.c_uint64()
        abi.check(self._lib.pbrtgpu_server_submit_render(self._h, scene._h, C.byref(renderer._cam),
                                                         C.byref(renderer._smp), ptr, C.byref(t)), self._lib)
        self._keep[t.value] = (scene, renderer, out)
        return t.value

    def submit_query(self, bvh: GpuBVHAccel, rays, any_hit: bool = False, out=None) -> int:
        ptr, n, keep = _ray_buffer(rays)
        if out is None:
            if _is_torch(rays) and rays.is_cuda:
                torch = _torch()
                out = (torch.empty((n,), dtype=torch.uint8, device=rays.device) if any_hit
                       else torch.empty((n, 4), dtype=torch.float32, device=rays.device))
            else:
                out = np.empty(n, dtype=np.uint8 if any_hit else abi.HIT_DTYPE)
        optr = C.c_void_p(out.data_ptr() if _is_torch(out) else out.ctypes.data)
        t = C.c_uint64()
        abi.check(self._lib.pbrtgpu_server_submit_query(self._h, bvh._h, ptr, n, None if any_hit else optr,
                                                        optr if any_hit else None, C.byref(t)), self._lib)
        self._keep[t.value] = (bvh, keep, out)
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0):
        """The request's output once it has completed (raises PbrtError with
        the request's status if it failed)."""
        st = C.c_int32()
        abi.check(self._lib.pbrtgpu_server_wait(self._h, ticket, float(timeout), C.byref(st)), self._lib)
        out = self._keep.pop(ticket)[-1]
        if st.value:
            raise abi.PbrtError(st.value, f"request {ticket} failed")
        return out

    def drain(self) -> None:
        abi.check(self._lib.pbrtgpu_server_drain(self._h), self._lib)

    def stats(self) -> dict:
        s = abi.PbrtServerStats()
        abi.check(self._lib.pbrtgpu_server_stats(self._h, C.byref(s)), self._lib)
        return {f: getattr(s, f) for f, _ in s._fields_}

    def reset_stats(self) -> None:
        abi.check(self._lib.pbrtgpu_server_reset_stats(self._h), self._lib)
