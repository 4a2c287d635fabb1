"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module.  It builds ``liboracle.so`` on first use.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
from pbrt_rust_gb300 import abi  # noqa: E402  (shared struct layouts only)
from pbrt_rust_gb300.scene import SceneDescription  # noqa: E402

import importlib.util as _ilu  # noqa: E402

_spec = _ilu.spec_from_file_location("pbrt_oracle_build", HERE / "build.py")
_build = _ilu.module_from_spec(_spec)
_spec.loader.exec_module(_build)

_lib = None
_P = C.c_void_p


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        lib = C.CDLL(str(path))
        sig = {
            "oracle_bvh_create": (C.c_int, [C.POINTER(abi.PbrtShapeDesc), C.c_uint32, C.c_uint32, C.c_char_p,
                                            C.POINTER(_P)]),
            "oracle_bvh_create_desc": (C.c_int, [C.POINTER(abi.PbrtSceneDesc), C.POINTER(_P)]),
            "oracle_bvh_destroy": (None, [_P]),
            "oracle_bvh_num_nodes": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
            "oracle_bvh_num_primitives": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
            "oracle_bvh_depth": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
            "oracle_bvh_get_nodes": (C.c_int, [_P, _P, C.c_uint32]),
            "oracle_bvh_get_primitive_order": (C.c_int, [_P, _P, C.c_uint32]),
            "oracle_bvh_world_bound": (C.c_int, [_P, _P, _P]),
            "oracle_bvh_triangle": (C.c_int, [_P, C.c_uint32, _P]),
            "oracle_intersect": (C.c_int, [_P, _P, C.c_uint32, _P, _P, C.c_int]),
            "oracle_intersect_p": (C.c_int, [_P, _P, C.c_uint32, _P, _P, C.c_int]),
            "oracle_count_first_hit": (C.c_int, [_P, _P, C.c_uint32, _P, _P, C.c_int]),
            "oracle_render": (C.c_int, [C.POINTER(abi.PbrtSceneDesc), C.POINTER(abi.PbrtCameraDesc),
                                        C.POINTER(abi.PbrtSamplerDesc), _P, C.c_int, C.c_uint32, C.c_uint32, _P]),
            "oracle_scene_create": (C.c_int, [C.POINTER(abi.PbrtSceneDesc), C.POINTER(_P)]),
            "oracle_scene_destroy": (None, [_P]),
            "oracle_scene_render": (C.c_int, [_P, C.POINTER(abi.PbrtCameraDesc), C.POINTER(abi.PbrtSamplerDesc), _P,
                                              C.c_int, C.c_uint32, C.c_uint32, _P]),
            "oracle_task_samples": (C.c_int, [C.POINTER(abi.PbrtSceneDesc), C.POINTER(abi.PbrtCameraDesc),
                                              C.POINTER(abi.PbrtSamplerDesc), C.c_uint32, _P, C.c_uint64, _P, _P]),
            "oracle_quadratic": (C.c_int, [C.c_float, C.c_float, C.c_float, _P, _P]),
            "oracle_partition_by_f32": (None, [_P, C.c_uint32]),
            "oracle_partition_by_i64": (None, [_P, C.c_uint32]),
            "oracle_crop_window": (None, [C.c_uint32, C.c_uint32, C.c_float, _P]),
            "oracle_sub_window": (None, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint32, C.c_uint32, _P]),
            "oracle_bbox_intersect": (C.c_int, [_P, _P, _P, _P]),
            "oracle_bbox_metrics": (None, [_P, _P, _P, _P]),
            "oracle_triangle_intersect": (C.c_int, [_P, _P, _P]),
            "oracle_quadric_intersect": (C.c_int, [C.c_int, C.POINTER(abi.PbrtTransform), C.c_float, C.c_float,
                                                   C.c_float, C.c_float, _P, C.c_int, _P]),
            "oracle_sphere_intersect": (C.c_int, [C.POINTER(abi.PbrtTransform), C.c_float, C.c_float, C.c_float,
                                                  C.c_float, _P, C.c_int, _P]),
            "oracle_matrix_invert": (C.c_int, [_P, _P]),
            "oracle_look_at": (None, [_P, _P, _P, C.POINTER(abi.PbrtTransform)]),
            "oracle_projection": (None, [C.c_uint32, C.c_uint32, C.POINTER(abi.PbrtTransform), _P,
                                         C.POINTER(abi.PbrtTransform)]),
            "oracle_perspective": (None, [C.c_float, C.POINTER(abi.PbrtTransform)]),
            "oracle_transform_point": (None, [C.POINTER(abi.PbrtTransform), _P, _P]),
            "oracle_transform_vector": (None, [C.POINTER(abi.PbrtTransform), _P, _P]),
            "oracle_film_extents": (None, [C.c_uint32, C.c_uint32, _P, C.c_float, C.c_float, _P, _P]),
            "oracle_filter_eval": (C.c_float, [C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                               C.c_float]),
            "oracle_rng_words": (None, [C.c_uint64, C.c_uint64, C.c_uint32, _P]),
            "oracle_chacha_blocks": (None, [_P, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, _P]),
            "oracle_rng_key": (None, [C.c_uint64, _P]),
            "oracle_rng_floats": (None, [C.c_uint64, C.c_uint32, _P]),
            "oracle_rng_uints": (None, [C.c_uint64, C.c_uint32, _P]),
            "oracle_rng_shuffle_i64": (None, [C.c_uint64, _P, C.c_uint32, C.c_uint32, C.c_uint32]),
            "oracle_rng_permutation": (None, [C.c_uint64, _P, C.c_uint32]),
            "oracle_stratified": (None, [C.c_uint64, _P, C.c_uint32, _P]),
            "oracle_latin_hypercube": (None, [C.c_uint64, C.c_uint32, C.c_uint32, _P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


class OracleBVH:
    """BVHAccelerator::new restated on the CPU."""

    def __init__(self, prims, max_prims: int = 4, split_method: str = "sah"):
        from pbrt_rust_gb300.scene import Primitive
        self.lib = load()
        prims = [p if isinstance(p, Primitive) else Primitive.simple(p) for p in prims]
        self.desc = SceneDescription(prims, [], max_prims, split_method, aggregate_only=True)
        h = C.c_void_p()
        if self.desc.definitions:  # instances (TransformedPrimitive) among the primitives
            st = self.lib.oracle_bvh_create_desc(C.byref(self.desc.desc), C.byref(h))
        else:
            st = self.lib.oracle_bvh_create(self.desc.shapes, self.desc.desc.n_shapes, int(max_prims),
                                            split_method.encode(), C.byref(h))
        if st:
            raise abi.PbrtError(st, "oracle BVH build failed")
        self.h = h

    def __del__(self):
        try:
            if self.h:
                self.lib.oracle_bvh_destroy(self.h)
        except Exception:
            pass

    def _u32(self, fn) -> int:
        v = C.c_uint32()
        fn(self.h, C.byref(v))
        return v.value

    def num_nodes(self) -> int:
        return self._u32(self.lib.oracle_bvh_num_nodes)

    def num_primitives(self) -> int:
        return self._u32(self.lib.oracle_bvh_num_primitives)

    def depth(self) -> int:
        return self._u32(self.lib.oracle_bvh_depth)

    def nodes(self) -> np.ndarray:
        n = self.num_nodes()
        out = np.zeros(n, dtype=abi.NODE_DTYPE)
        self.lib.oracle_bvh_get_nodes(self.h, _ptr(out), n)
        return out

    def primitive_order(self) -> np.ndarray:
        n = self.num_primitives()
        out = np.zeros(n, dtype=np.uint32)
        self.lib.oracle_bvh_get_primitive_order(self.h, _ptr(out), n)
        return out

    def world_bound(self):
        lo = np.zeros(3, np.float32)
        hi = np.zeros(3, np.float32)
        self.lib.oracle_bvh_world_bound(self.h, _ptr(lo), _ptr(hi))
        return lo, hi

    def triangle(self, prim: int) -> np.ndarray:
        out = np.zeros(9, np.float32)
        if self.lib.oracle_bvh_triangle(self.h, prim, _ptr(out)):
            raise ValueError("not a triangle")
        return out.reshape(3, 3)

    def intersect(self, rays: np.ndarray, nthreads: int | None = None, counters: bool = False):
        rays = np.ascontiguousarray(rays)
        n = rays.shape[0]
        hits = np.zeros(n, dtype=abi.HIT_DTYPE)
        cnt = np.zeros(3, np.uint64)
        self.lib.oracle_intersect(self.h, _ptr(rays), n, _ptr(hits), _ptr(cnt), nthreads or default_threads())
        return (hits, cnt) if counters else hits

    def first_hit_counts(self, rays: np.ndarray, nthreads: int | None = None):
        """(answers, counters) of the any-hit walk stopped at its first
        accepted primitive: the early-exit work; the answers equal
        intersect_p's."""
        rays = np.ascontiguousarray(rays)
        n = rays.shape[0]
        occ = np.zeros(n, dtype=np.uint8)
        cnt = np.zeros(3, np.uint64)
        self.lib.oracle_count_first_hit(self.h, _ptr(rays), n, _ptr(occ), _ptr(cnt), nthreads or default_threads())
        return occ, cnt

    def intersect_p(self, rays: np.ndarray, nthreads: int | None = None, counters: bool = False):
        rays = np.ascontiguousarray(rays)
        n = rays.shape[0]
        occ = np.zeros(n, dtype=np.uint8)
        cnt = np.zeros(3, np.uint64)
        self.lib.oracle_intersect_p(self.h, _ptr(rays), n, _ptr(occ), _ptr(cnt), nthreads or default_threads())
        return (occ, cnt) if counters else occ


def render(desc: SceneDescription, camera, sampler, num_tasks: int, nthreads: int | None = None,
           task_lo: int = 0, task_hi: int | None = None, stats: bool = False):
    """SamplerRenderer::render restated on the CPU; returns (h, w, 3) RGB."""
    lib = load()
    cam = camera.to_abi()
    smp = sampler.to_abi(num_tasks)
    x0, x1, y0, y1 = camera.film.pixel_extent()
    rgb = np.zeros((y1 - y0, x1 - x0, 3), np.float32)
    st_arr = np.zeros(8, np.uint64)
    st = lib.oracle_render(C.byref(desc.desc), C.byref(cam), C.byref(smp), _ptr(rgb), nthreads or default_threads(),
                           task_lo, num_tasks if task_hi is None else task_hi, _ptr(st_arr))
    if st:
        raise abi.PbrtError(st, "oracle render failed")
    return (rgb, st_arr) if stats else rgb


class OracleScene:
    """A scene built once by the oracle (BVH, shading tables), rendered many
    times: render() is the same SamplerRenderer::render restatement as the
    module-level render(), without the per-call scene build."""

    def __init__(self, desc: SceneDescription):
        self.lib = load()
        self.desc = desc  # keeps the description's arrays alive
        h = C.c_void_p()
        st = self.lib.oracle_scene_create(C.byref(desc.desc), C.byref(h))
        if st:
            raise abi.PbrtError(st, "oracle scene build failed")
        self.h = h

    def __del__(self):
        try:
            if self.h:
                self.lib.oracle_scene_destroy(self.h)
        except Exception:
            pass

    def render(self, camera, sampler, num_tasks: int, nthreads: int | None = None, task_lo: int = 0,
               task_hi: int | None = None):
        """Returns (rgb (h, w, 3), stats): stats as oracle_render's 8 words
        (camera rays, shadow rays, then nodes / triangles / analytic shapes
        tested by camera rays and by shadow rays)."""
        cam = camera.to_abi()
        smp = sampler.to_abi(num_tasks)
        x0, x1, y0, y1 = camera.film.pixel_extent()
        rgb = np.zeros((y1 - y0, x1 - x0, 3), np.float32)
        st_arr = np.zeros(8, np.uint64)
        st = self.lib.oracle_scene_render(self.h, C.byref(cam), C.byref(smp), _ptr(rgb),
                                          nthreads or default_threads(), task_lo,
                                          num_tasks if task_hi is None else task_hi, _ptr(st_arr))
        if st:
            raise abi.PbrtError(st, "oracle render failed")
        return rgb, st_arr


def task_samples(desc: SceneDescription, camera, sampler, num_tasks: int, task: int) -> np.ndarray:
    """Per-sample dump of one task (see oracle.h): (n, stride) float32."""
    lib = load()
    cam = camera.to_abi()
    smp = sampler.to_abi(num_tasks)
    cap = 1 << 26
    out = np.zeros(cap, np.float32)
    n = C.c_uint32()
    stride = C.c_uint32()
    st = lib.oracle_task_samples(C.byref(desc.desc), C.byref(cam), C.byref(smp), task, _ptr(out), cap,
                                 C.byref(n), C.byref(stride))
    if st:
        raise abi.PbrtError(st, "oracle task_samples failed")
    return out[: n.value * stride.value].reshape(n.value, stride.value).copy()
