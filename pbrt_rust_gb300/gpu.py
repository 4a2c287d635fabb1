"""The two drop-ins over the compiled library.

``GpuBVHAccel`` replaces the BVH aggregate (``Aggregate::bvh``,
src/primitive/aggregates/mod.rs:27-29; ``BVHAccelerator``,
src/primitive/aggregates/bvh.rs:328-422) behind the reference's
``Intersectable`` / ``HasBounds`` surface, batched over rays.

``GpuSamplerRenderer`` replaces ``SamplerRenderer``
(src/sampler_renderer.rs:25-213): same constructor arguments, ``render``
returns the film's linear RGB image.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .scene import (Camera, Primitive, SceneDescription, StratifiedSampler, default_num_tasks)


def _torch():
    try:
        import torch  # noqa: F401
        return torch
    except Exception:  # pragma: no cover - torch is optional for host buffers
        return None


def _is_torch(x) -> bool:
    t = _torch()
    return t is not None and isinstance(x, t.Tensor)


def _stream_handle(stream) -> C.c_void_p:
    if stream is None:
        t = _torch()
        if t is not None and t.cuda.is_available():
            return C.c_void_p(t.cuda.current_stream().cuda_stream)
        return C.c_void_p(0)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


def _ray_buffer(rays):
    """(pointer, n, keepalive) for a host ndarray of RAY_DTYPE / (n, 8) f32,
    or a (n, 8) float32 torch tensor (device or host)."""
    if _is_torch(rays):
        if rays.dtype != _torch().float32 or rays.dim() != 2 or rays.shape[1] != 8 or not rays.is_contiguous():
            raise ValueError("rays tensor must be a contiguous (n, 8) float32 tensor")
        return C.c_void_p(rays.data_ptr()), rays.shape[0], rays
    a = np.asarray(rays)
    if a.dtype == abi.RAY_DTYPE:
        a = np.ascontiguousarray(a)
        n = a.shape[0]
    else:
        a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1, 8)
        n = a.shape[0]
    return C.c_void_p(a.ctypes.data), n, a


class GpuBVHAccel:
    """BVHAccelerator on the device.  ``prims`` is a list of Primitive (or
    Shape); every mesh refines to its triangles in index order, and hit
    indices refer to that refined list."""

    def __init__(self, prims, max_prims: int = 4, split_method: str = "sah", _handle=None, _owner=None,
                 build_on_device: bool = False):
        """``build_on_device`` builds the tree with CUDA kernels (same
        result as the host build)."""
        self._lib = abi.load()
        self._owner = _owner
        if _handle is not None:
            self._h = _handle
            self._own = False
            self.desc = None
            return
        prims = [p if isinstance(p, Primitive) else Primitive.simple(p) for p in prims]
        self.desc = SceneDescription(prims, [], max_prims, split_method, aggregate_only=True)
        h = C.c_void_p()
        flags = abi.BUILD_ON_DEVICE if build_on_device else 0
        if self.desc.definitions:  # TransformedPrimitive instances among the primitives
            self.desc.desc.build_flags = flags
            abi.check(self._lib.pbrtgpu_bvh_create_desc(C.byref(self.desc.desc), C.byref(h)), self._lib)
        else:
            abi.check(self._lib.pbrtgpu_bvh_create_ex(self.desc.shapes, self.desc.desc.n_shapes, int(max_prims),
                                                      split_method.encode(), flags, C.byref(h)),
                      self._lib)
        self._h = h
        self._own = True

    def close(self) -> None:
        if getattr(self, "_own", False) and self._h:
            self._lib.pbrtgpu_bvh_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # HasBounds::world_bound (bvh.rs:365-373)
    def world_bound(self) -> tuple[np.ndarray, np.ndarray]:
        lo = (C.c_float * 3)()
        hi = (C.c_float * 3)()
        abi.check(self._lib.pbrtgpu_bvh_world_bound(self._h, lo, hi), self._lib)
        return np.array(lo[:], dtype=np.float32), np.array(hi[:], dtype=np.float32)

    def _u32(self, fn) -> int:
        v = C.c_uint32()
        abi.check(fn(self._h, C.byref(v)), self._lib)
        return v.value

    def num_primitives(self) -> int:
        return self._u32(self._lib.pbrtgpu_bvh_num_primitives)

    def num_nodes(self) -> int:
        return self._u32(self._lib.pbrtgpu_bvh_num_nodes)

    def device_bytes(self) -> int:
        """Device memory the aggregate keeps resident."""
        v = C.c_uint64()
        abi.check(self._lib.pbrtgpu_bvh_device_bytes(self._h, C.byref(v)), self._lib)
        return v.value

    def depth(self) -> int:
        return self._u32(self._lib.pbrtgpu_bvh_depth)

    def nodes(self) -> np.ndarray:
        n = self.num_nodes()
        out = np.zeros(n, dtype=abi.NODE_DTYPE)
        abi.check(self._lib.pbrtgpu_bvh_get_nodes(self._h, C.c_void_p(out.ctypes.data), n), self._lib)
        return out

    def primitive_order(self) -> np.ndarray:
        n = self.num_primitives()
        out = np.zeros(n, dtype=np.uint32)
        abi.check(self._lib.pbrtgpu_bvh_get_primitive_order(self._h, abi.u32p(out), n), self._lib)
        return out

    # Intersectable::intersect over a batch (bvh.rs:375-422)
    def intersect(self, rays, out=None, stream=None):
        """Closest hits.  Host rays -> HIT_DTYPE ndarray; a (n, 8) float32
        CUDA tensor -> (n, 4) float32 CUDA tensor (prim bits, t, b1, b2),
        queued on `stream` (default: torch's current stream)."""
        ptr, n, keep = _ray_buffer(rays)
        if _is_torch(rays):
            torch = _torch()
            if out is None:
                out = torch.empty((n, 4), dtype=torch.float32, device=rays.device)
            optr = C.c_void_p(out.data_ptr())
        else:
            if out is None:
                out = np.empty(n, dtype=abi.HIT_DTYPE)
            optr = C.c_void_p(out.ctypes.data)
        abi.check(self._lib.pbrtgpu_intersect(self._h, ptr, n, optr, _stream_handle(stream)), self._lib)
        del keep
        return out

    # Intersectable::intersect_p (src/intersection.rs:61-66)
    def intersect_p(self, rays, out=None, stream=None):
        ptr, n, keep = _ray_buffer(rays)
        if _is_torch(rays):
            torch = _torch()
            if out is None:
                out = torch.empty((n,), dtype=torch.uint8, device=rays.device)
            optr = C.c_void_p(out.data_ptr())
        else:
            if out is None:
                out = np.empty(n, dtype=np.uint8)
            optr = C.c_void_p(out.ctypes.data)
        abi.check(self._lib.pbrtgpu_intersect_p(self._h, ptr, n, optr, _stream_handle(stream)), self._lib)
        del keep
        return out


class GpuScene:
    """Scene::new_with (src/scene.rs:31-39) on the device: the aggregate
    plus materials and lights."""

    def __init__(self, prims: list[Primitive], lights: list = (), max_prims: int = 4, split_method: str = "sah",
                 build_on_device: bool = False):
        self._lib = abi.load()
        self.desc = SceneDescription(prims, lights, max_prims, split_method)
        self.desc.desc.build_flags = abi.BUILD_ON_DEVICE if build_on_device else 0
        h = C.c_void_p()
        abi.check(self._lib.pbrtgpu_scene_create(C.byref(self.desc.desc), C.byref(h)), self._lib)
        self._h = h

    def aggregate(self) -> GpuBVHAccel:
        b = C.c_void_p()
        abi.check(self._lib.pbrtgpu_scene_bvh(self._h, C.byref(b)), self._lib)
        return GpuBVHAccel(None, _handle=b, _owner=self)

    def device_bytes(self) -> int:
        """Device memory the scene keeps resident (BVH + shading tables)."""
        v = C.c_uint64()
        abi.check(self._lib.pbrtgpu_scene_device_bytes(self._h, C.byref(v)), self._lib)
        return v.value

    def close(self) -> None:
        if self._h:
            self._lib.pbrtgpu_scene_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuSamplerRenderer:
    """SamplerRenderer::new(sampler, camera, surface, volume)
    (src/sampler_renderer.rs:37-54).  The surface integrator is the
    direct-lighting light loop; ``num_tasks`` fixes the reference's task
    split (and so its random streams)."""

    def __init__(self, sampler: StratifiedSampler, camera: Camera, surface_integrator=None,
                 volume_integrator=None, num_tasks: int | None = None):
        self._lib = abi.load()
        self.sampler = sampler
        self.camera = camera
        self.num_tasks = num_tasks if num_tasks is not None else default_num_tasks(camera.film.x_res,
                                                                                  camera.film.y_res)
        self._cam = camera.to_abi()
        self._smp = sampler.to_abi(self.num_tasks)

    def pixel_extent(self) -> tuple[int, int, int, int]:
        ext = (C.c_int32 * 4)()
        abi.check(self._lib.pbrtgpu_film_pixel_extent(C.byref(self._cam), ext), self._lib)
        return tuple(ext[:])

    def render(self, scene: GpuScene, out=None, stream=None, tasks: tuple[int, int] | None = None):
        """Renderer::render: returns (h, w, 3) float32 linear RGB (a numpy
        array, or `out` if given: a host array or a CUDA tensor).  With
        ``tasks=(lo, hi)`` only those tasks of the split are rendered and the
        pixels of the others are 0 (one shard of a frame)."""
        x0, x1, y0, y1 = self.pixel_extent()
        shape = (y1 - y0, x1 - x0, 3)
        if out is None:
            out = np.zeros(shape, dtype=np.float32)
        if _is_torch(out):
            ptr = C.c_void_p(out.data_ptr())
        else:
            if out.shape != shape or out.dtype != np.float32 or not out.flags.c_contiguous:
                raise ValueError(f"out must be a contiguous float32 array of shape {shape}")
            ptr = C.c_void_p(out.ctypes.data)
        if tasks is None:
            st = self._lib.pbrtgpu_render(scene._h, C.byref(self._cam), C.byref(self._smp), ptr,
                                          _stream_handle(stream))
        else:
            st = self._lib.pbrtgpu_render_tasks(scene._h, C.byref(self._cam), C.byref(self._smp), int(tasks[0]),
                                                int(tasks[1]), ptr, _stream_handle(stream))
        abi.check(st, self._lib)
        if self.camera.film.filename and tasks is None:  # sampler_renderer.rs:181: write_image at the end
            write_image(out, self.camera.film.filename)
        return out


def write_image(rgb, path: str) -> None:
    """Film::write_image (src/camera/film.rs:316-354, write_img :15-33):
    .png / .ppm with write_img's 8-bit values, .pfm with the linear floats;
    `rgb` is an (h, w, 3) float32 host array or CUDA tensor."""
    if _is_torch(rgb):
        rgb = rgb.detach().cpu().numpy()
    a = np.ascontiguousarray(rgb, dtype=np.float32)
    if a.ndim != 3 or a.shape[2] != 3:
        raise ValueError("rgb must have shape (height, width, 3)")
    lib = abi.load()
    abi.check(lib.pbrtgpu_write_image(C.c_void_p(a.ctypes.data), a.shape[1], a.shape[0], str(path).encode()), lib)


def image_bytes(rgb) -> np.ndarray:
    """The 8-bit values write_img stores for `rgb` (film.rs:22-24)."""
    if _is_torch(rgb):
        rgb = rgb.detach().cpu().numpy()
    a = np.ascontiguousarray(rgb, dtype=np.float32)
    out = np.empty(a.shape, np.uint8)
    lib = abi.load()
    abi.check(lib.pbrtgpu_image_bytes(C.c_void_p(a.ctypes.data), a.shape[1], a.shape[0],
                                      C.c_void_p(out.ctypes.data)), lib)
    return out
