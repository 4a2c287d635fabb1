"""Batched multi-scene rendering and ray queries (``pbrtgpu_batch_*``).

A ``GpuBatch`` collects render jobs (a ``GpuScene`` with a
``GpuSamplerRenderer``'s camera and sampler, exactly what
``GpuSamplerRenderer.render`` takes) and ray-query jobs (a ``GpuBVHAccel``
and a ray array, as for ``intersect`` / ``intersect_p``) over any number of
scenes, and runs them together: every wavefront stage is one launch over the
items of all jobs, the traversal stages are persistent kernels fed by a
device work counter, and the stage sequence replays as one CUDA graph.  Each
job's output is the one the single-job call gives, bit for bit.

The reference has no such mode: ``SamplerRenderer::render``
(src/sampler_renderer.rs:146-176) renders one scene per call.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .gpu import GpuBVHAccel, GpuSamplerRenderer, GpuScene, _is_torch, _ray_buffer, _stream_handle, _torch

_KERNEL = {"pair": abi.TRACE_KERNELS["plain"], "wide": abi.TRACE_KERNELS["w4"]}
_KERNEL_NAME = {v: k for k, v in _KERNEL.items()}


def limits(max_jobs: int = 64, max_tasks: int = 4096, max_samples: int = 1 << 22, max_light_samples: int | None = None,
           max_film_pixels: int = 1 << 20, max_query_rays: int = 0) -> abi.PbrtBatchLimits:
    L = abi.PbrtBatchLimits()
    L.max_jobs = max_jobs
    L.max_tasks = max_tasks
    L.max_samples = max_samples
    L.max_light_samples = 2 * max_samples if max_light_samples is None else max_light_samples
    L.max_film_pixels = max_film_pixels
    L.max_query_rays = max_query_rays
    return L


def batch_bytes(**kw) -> tuple[int, int]:
    """(device bytes, pinned host bytes) a batch with these limits allocates."""
    lib = abi.load()
    d, h = C.c_uint64(), C.c_uint64()
    abi.check(lib.pbrtgpu_batch_bytes(C.byref(limits(**kw)), C.byref(d), C.byref(h)), lib)
    return d.value, h.value


class GpuBatch:
    """Limits (keyword arguments of ``limits``) fix the device memory the
    batch holds; a job beyond them is refused with PBRT_ERR_BUDGET."""

    def __init__(self, **kw):
        self._lib = abi.load()
        self.limits = limits(**kw)
        h = C.c_void_p()
        abi.check(self._lib.pbrtgpu_batch_create(C.byref(self.limits), C.byref(h)), self._lib)
        self._h = h
        self._keep = []   # host buffers and handles the current jobs use
        self._outs = []

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.pbrtgpu_batch_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_render(self, scene: GpuScene, renderer: GpuSamplerRenderer, out=None) -> int:
        """Queues renderer.render(scene); the image goes to `out` (host array
        or CUDA tensor of the film's shape, allocated on the host if None) and
        is also returned by ``wait``."""
        x0, x1, y0, y1 = renderer.pixel_extent()
        shape = (y1 - y0, x1 - x0, 3)
        if out is None:
            out = np.zeros(shape, dtype=np.float32)
        ptr = C.c_void_p(out.data_ptr() if _is_torch(out) else out.ctypes.data)
        job = C.c_uint32()
        abi.check(self._lib.pbrtgpu_batch_add_render(self._h, scene._h, C.byref(renderer._cam), C.byref(renderer._smp),
                                                     ptr, C.byref(job)), self._lib)
        self._keep += [scene, renderer, out]
        self._outs.append(out)
        return job.value

    def add_query(self, bvh: GpuBVHAccel, rays, any_hit: bool = False, out=None) -> int:
        """Queues bvh.intersect(rays) (or intersect_p with any_hit)."""
        ptr, n, keep = _ray_buffer(rays)
        if out is None:
            if _is_torch(rays) and rays.is_cuda:
                torch = _torch()
                out = (torch.empty((n,), dtype=torch.uint8, device=rays.device) if any_hit
                       else torch.empty((n, 4), dtype=torch.float32, device=rays.device))
            else:
                out = np.empty(n, dtype=np.uint8 if any_hit else abi.HIT_DTYPE)
        optr = C.c_void_p(out.data_ptr() if _is_torch(out) else out.ctypes.data)
        job = C.c_uint32()
        abi.check(self._lib.pbrtgpu_batch_add_query(self._h, bvh._h, ptr, n, None if any_hit else optr,
                                                    optr if any_hit else None, C.byref(job)), self._lib)
        self._keep += [bvh, keep, out]
        self._outs.append(out)
        return job.value

    def launch(self, stream=None) -> None:
        abi.check(self._lib.pbrtgpu_batch_launch(self._h, _stream_handle(stream)), self._lib)

    def poll(self) -> bool:
        d = C.c_int32()
        abi.check(self._lib.pbrtgpu_batch_poll(self._h, C.byref(d)), self._lib)
        return bool(d.value)

    def wait(self, check: bool = True):
        """Waits for the launch and empties the batch.  Returns the jobs'
        outputs in job order (and raises on the first failed job unless
        check is False, then returns (outputs, statuses))."""
        n = len(self._outs)
        st = (C.c_int32 * max(n, 1))()
        r = self._lib.pbrtgpu_batch_wait(self._h, st)
        outs = self._outs
        self._outs, self._keep = [], []
        if check:
            abi.check(r, self._lib)
            return outs
        return outs, list(st[:n])

    def run(self, stream=None):
        self.launch(stream)
        return self.wait()

    @property
    def tuning(self) -> dict:
        t = abi.PbrtBatchTuning()
        abi.check(self._lib.pbrtgpu_batch_get_tuning(self._h, C.byref(t)), self._lib)
        d = t.as_dict()
        d["extend_kernel"] = _KERNEL_NAME[d["extend_kernel"]]
        d["shadow_kernel"] = _KERNEL_NAME[d["shadow_kernel"]]
        return d

    def set_tuning(self, **kw) -> None:
        d = dict(self.tuning, **kw)
        t = abi.PbrtBatchTuning()
        for k, v in d.items():
            setattr(t, k, _KERNEL[v] if k in ("extend_kernel", "shadow_kernel") else int(v))
        abi.check(self._lib.pbrtgpu_batch_set_tuning(self._h, C.byref(t)), self._lib)

    def autotune(self, stream=None, repeats: int = 3) -> tuple[dict, float]:
        """Times the queued jobs under candidate tunings, keeps the fastest;
        the jobs stay queued."""
        t = abi.PbrtBatchTuning()
        ms = C.c_float()
        abi.check(self._lib.pbrtgpu_batch_autotune(self._h, _stream_handle(stream), repeats, C.byref(t),
                                                   C.byref(ms)), self._lib)
        return self.tuning, ms.value

    def stats(self) -> dict:
        s = abi.PbrtBatchStats()
        abi.check(self._lib.pbrtgpu_batch_stats(self._h, C.byref(s)), self._lib)
        return {f: getattr(s, f) for f, _ in s._fields_ if f != "pad"}
