"""ctypes mirror of ``include/pbrt_gpu.h`` and the library loader.

The loader raises if the compiled library is missing or cannot be loaded:
there is no CPU fallback behind this package.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libpbrt_gb300.so"

PBRT_OK = 0
STATUS_NAMES = {
    0: "PBRT_OK", 1: "PBRT_ERR_INVALID_ARGUMENT", 2: "PBRT_ERR_CUDA", 3: "PBRT_ERR_OUT_OF_MEMORY",
    4: "PBRT_ERR_UNSUPPORTED", 5: "PBRT_ERR_BUILD", 6: "PBRT_ERR_STACK_OVERFLOW", 7: "PBRT_ERR_BUDGET",
    8: "PBRT_ERR_TIMEOUT", 9: "PBRT_ERR_NAN", 10: "PBRT_ERR_NO_DEVICE", 11: "PBRT_ERR_CANCELLED",
}
PBRT_ERR_INVALID_ARGUMENT = 1
PBRT_ERR_CUDA = 2
PBRT_ERR_OUT_OF_MEMORY = 3
PBRT_ERR_UNSUPPORTED = 4
PBRT_ERR_BUILD = 5
PBRT_ERR_STACK_OVERFLOW = 6
PBRT_ERR_BUDGET = 7
PBRT_ERR_TIMEOUT = 8
PBRT_ERR_NAN = 9
PBRT_ERR_NO_DEVICE = 10
PBRT_ERR_CANCELLED = 11

ABI_VERSION = 2  # PBRT_GPU_ABI_VERSION

SHAPE_TRIANGLE_MESH = 0
SHAPE_SPHERE = 1
SHAPE_DISK = 2
SHAPE_CYLINDER = 3
SHAPE_INSTANCE = 4
LIGHT_POINT = 0
LIGHT_DIFFUSE_AREA = 1
SPLIT_METHODS = {"sah": 0, "middle": 1, "equal": 2}
BUILD_ON_DEVICE = 1

# 32-byte ray and 16-byte hit records (PbrtRay / PbrtHit).
RAY_DTYPE = np.dtype([("o", "<f4", 3), ("tmin", "<f4"), ("d", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("prim", "<i4"), ("t", "<f4"), ("b1", "<f4"), ("b2", "<f4")])
FLT_MAX = float(np.finfo(np.float32).max)


class PbrtError(RuntimeError):
    """A failing status from the library; ``status`` holds the code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class PbrtTransform(C.Structure):
    _fields_ = [("m", C.c_float * 16), ("m_inv", C.c_float * 16)]


class PbrtShapeDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("reverse_orientation", C.c_int32), ("object_to_world", PbrtTransform),
        ("points", C.POINTER(C.c_float)), ("n_points", C.c_uint32),
        ("indices", C.POINTER(C.c_uint32)), ("n_indices", C.c_uint32),
        ("radius", C.c_float), ("z0", C.c_float), ("z1", C.c_float), ("phi_max_deg", C.c_float),
        ("height", C.c_float), ("inner_radius", C.c_float),
        ("instance", C.c_int32),
        ("material", C.c_int32), ("area_light", C.c_int32),
    ]


class PbrtInstanceDesc(C.Structure):
    _fields_ = [("shapes", C.POINTER(PbrtShapeDesc)), ("n_shapes", C.c_uint32)]


class PbrtMaterialDesc(C.Structure):
    _fields_ = [("kd", C.c_float * 3), ("sigma", C.c_float)]


class PbrtLightDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("light_to_world", PbrtTransform), ("spectrum", C.c_float * 3),
                ("shape", C.c_int32)]


class PbrtSceneDesc(C.Structure):
    _fields_ = [
        ("shapes", C.POINTER(PbrtShapeDesc)), ("n_shapes", C.c_uint32),
        ("materials", C.POINTER(PbrtMaterialDesc)), ("n_materials", C.c_uint32),
        ("lights", C.POINTER(PbrtLightDesc)), ("n_lights", C.c_uint32),
        ("max_prims_in_node", C.c_uint32), ("split_method", C.c_int32), ("build_flags", C.c_uint32),
        ("instances", C.POINTER(PbrtInstanceDesc)), ("n_instances", C.c_uint32),
    ]


class PbrtCameraDesc(C.Structure):
    _fields_ = [
        ("camera_to_world", PbrtTransform), ("fov_deg", C.c_float), ("screen_window", C.c_float * 4),
        ("lens_radius", C.c_float), ("focal_distance", C.c_float),
        ("shutter_open", C.c_float), ("shutter_close", C.c_float),
        ("x_res", C.c_uint32), ("y_res", C.c_uint32), ("crop_window", C.c_float * 4),
        ("filter_x_width", C.c_float), ("filter_y_width", C.c_float),
        ("filter_kind", C.c_int32), ("filter_p0", C.c_float), ("filter_p1", C.c_float),
    ]


class PbrtSamplerDesc(C.Structure):
    _fields_ = [
        ("x_start", C.c_int32), ("x_end", C.c_int32), ("y_start", C.c_int32), ("y_end", C.c_int32),
        ("x_samples", C.c_uint32), ("y_samples", C.c_uint32), ("jitter", C.c_int32),
        ("shutter_open", C.c_float), ("shutter_close", C.c_float), ("num_tasks", C.c_uint32),
    ]


class PbrtTraceConfig(C.Structure):
    _fields_ = [("kernel", C.c_int32), ("refill", C.c_uint32), ("min_blocks", C.c_uint32),
                ("render_kernel", C.c_int32), ("reorder", C.c_uint32), ("chunk", C.c_uint32)]


TRACE_KERNELS = {"plain": 0, "pt": 1, "w4": 2, "w4pt": 3, "w4spec": 4, "packet": 5}
FILTERS = {"box": 0, "triangle": 1, "gaussian": 2, "mitchell": 3, "lanczos": 4}


class PbrtBatchLimits(C.Structure):
    _fields_ = [("max_jobs", C.c_uint32), ("max_tasks", C.c_uint32), ("max_samples", C.c_uint64),
                ("max_light_samples", C.c_uint64), ("max_film_pixels", C.c_uint64), ("max_query_rays", C.c_uint64)]


class PbrtBatchTuning(C.Structure):
    _fields_ = [("extend_kernel", C.c_int32), ("shadow_kernel", C.c_int32), ("block", C.c_uint32),
                ("stack", C.c_uint32), ("chunk", C.c_uint32), ("refill", C.c_uint32), ("refill_shadow", C.c_uint32),
                ("use_graph", C.c_uint32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class PbrtServerConfig(C.Structure):
    _fields_ = [("slots", C.c_uint32), ("use_tuning", C.c_uint32), ("limits", PbrtBatchLimits),
                ("tuning", PbrtBatchTuning), ("pool_bytes", C.c_uint64)]


class PbrtServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("batches", C.c_uint64), ("mean_batch_requests", C.c_double), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("max_ms", C.c_double), ("span_s", C.c_double),
                ("requests_per_s", C.c_double), ("pool_bytes", C.c_uint64), ("slot_bytes", C.c_uint64),
                ("resident_bytes", C.c_uint64), ("resident_count", C.c_uint64), ("deferred", C.c_uint64),
                ("refused", C.c_uint64)]


class PbrtBatchStats(C.Structure):
    _fields_ = [("jobs", C.c_uint32), ("kernels", C.c_uint32), ("samples", C.c_uint64),
                ("light_samples", C.c_uint64), ("film_pixels", C.c_uint64), ("query_rays", C.c_uint64),
                ("graph", C.c_uint32), ("pad", C.c_uint32)]


class PbrtPackedNode(C.Structure):
    _fields_ = [("lo", C.c_float * 3), ("hi", C.c_float * 3), ("is_leaf", C.c_int32), ("offset", C.c_uint32),
                ("count", C.c_uint32)]


NODE_DTYPE = np.dtype([("lo", "<f4", 3), ("hi", "<f4", 3), ("is_leaf", "<i4"), ("offset", "<u4"),
                       ("count", "<u4")])
assert NODE_DTYPE.itemsize == C.sizeof(PbrtPackedNode)

# Every symbol include/pbrt_gpu.h declares, with its ctypes signature.
_P = C.c_void_p
_U32P = C.POINTER(C.c_uint32)
_F3 = C.POINTER(C.c_float)
SIGNATURES = {
    "pbrtgpu_abi_version": (C.c_int, []),
    "pbrtgpu_status_str": (C.c_char_p, [C.c_int]),
    "pbrtgpu_last_error": (C.c_char_p, []),
    "pbrtgpu_bvh_create": (C.c_int, [C.POINTER(PbrtShapeDesc), C.c_uint32, C.c_uint32, C.c_char_p,
                                     C.POINTER(_P)]),
    "pbrtgpu_bvh_create_ex": (C.c_int, [C.POINTER(PbrtShapeDesc), C.c_uint32, C.c_uint32, C.c_char_p, C.c_uint32,
                                        C.POINTER(C.c_void_p)]),
    "pbrtgpu_bvh_create_desc": (C.c_int, [C.POINTER(PbrtSceneDesc), C.POINTER(C.c_void_p)]),
    "pbrtgpu_bvh_destroy": (None, [_P]),
    "pbrtgpu_bvh_world_bound": (C.c_int, [_P, _F3, _F3]),
    "pbrtgpu_bvh_num_primitives": (C.c_int, [_P, _U32P]),
    "pbrtgpu_bvh_device_bytes": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "pbrtgpu_bvh_num_nodes": (C.c_int, [_P, _U32P]),
    "pbrtgpu_bvh_depth": (C.c_int, [_P, _U32P]),
    "pbrtgpu_bvh_get_nodes": (C.c_int, [_P, _P, C.c_uint32]),
    "pbrtgpu_bvh_get_primitive_order": (C.c_int, [_P, _U32P, C.c_uint32]),
    "pbrtgpu_intersect": (C.c_int, [_P, _P, C.c_uint32, _P, _P]),
    "pbrtgpu_intersect_p": (C.c_int, [_P, _P, C.c_uint32, _P, _P]),
    "pbrtgpu_intersect_streamed": (C.c_int, [_P, _P, C.c_uint32, _P, _P, _P, C.c_uint32, _P]),
    "pbrtgpu_set_trace_config": (C.c_int, [C.POINTER(PbrtTraceConfig)]),
    "pbrtgpu_get_trace_config": (C.c_int, [C.POINTER(PbrtTraceConfig)]),
    "pbrtgpu_scene_create": (C.c_int, [C.POINTER(PbrtSceneDesc), C.POINTER(_P)]),
    "pbrtgpu_scene_destroy": (None, [_P]),
    "pbrtgpu_scene_device_bytes": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "pbrtgpu_scene_bvh": (C.c_int, [_P, C.POINTER(_P)]),
    "pbrtgpu_render": (C.c_int, [_P, C.POINTER(PbrtCameraDesc), C.POINTER(PbrtSamplerDesc), _P, _P]),
    "pbrtgpu_render_tasks": (C.c_int, [_P, C.POINTER(PbrtCameraDesc), C.POINTER(PbrtSamplerDesc), C.c_uint32,
                                       C.c_uint32, _P, _P]),
    "pbrtgpu_render_noalloc": (C.c_int, [_P, C.POINTER(PbrtCameraDesc), C.POINTER(PbrtSamplerDesc), _P, _P]),
    "pbrtgpu_film_pixel_extent": (C.c_int, [C.POINTER(PbrtCameraDesc), C.POINTER(C.c_int32)]),
    "pbrtgpu_chacha_blocks": (C.c_int, [_P, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, _P]),
    "pbrtgpu_rng_words": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, _P]),
    "pbrtgpu_filter_table": (C.c_int, [C.POINTER(PbrtCameraDesc), C.POINTER(C.c_float)]),
    "pbrtgpu_write_image": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_char_p]),
    "pbrtgpu_image_bytes": (C.c_int, [_P, C.c_uint32, C.c_uint32, _P]),
    "pbrtgpu_batch_bytes": (C.c_int, [C.POINTER(PbrtBatchLimits), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "pbrtgpu_batch_create": (C.c_int, [C.POINTER(PbrtBatchLimits), C.POINTER(C.c_void_p)]),
    "pbrtgpu_batch_destroy": (None, [_P]),
    "pbrtgpu_batch_add_render": (C.c_int, [_P, _P, C.POINTER(PbrtCameraDesc), C.POINTER(PbrtSamplerDesc), _P,
                                           C.POINTER(C.c_uint32)]),
    "pbrtgpu_batch_add_query": (C.c_int, [_P, _P, _P, C.c_uint32, _P, _P, C.POINTER(C.c_uint32)]),
    "pbrtgpu_batch_launch": (C.c_int, [_P, _P]),
    "pbrtgpu_batch_poll": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "pbrtgpu_batch_wait": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "pbrtgpu_batch_set_tuning": (C.c_int, [_P, C.POINTER(PbrtBatchTuning)]),
    "pbrtgpu_batch_get_tuning": (C.c_int, [_P, C.POINTER(PbrtBatchTuning)]),
    "pbrtgpu_batch_stats": (C.c_int, [_P, C.POINTER(PbrtBatchStats)]),
    "pbrtgpu_batch_autotune": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(PbrtBatchTuning), C.POINTER(C.c_float)]),
    "pbrtgpu_server_create": (C.c_int, [C.POINTER(PbrtServerConfig), C.POINTER(C.c_void_p)]),
    "pbrtgpu_server_admit": (C.c_int, [_P, _P, _P]),
    "pbrtgpu_server_release": (C.c_int, [_P, _P, _P]),
    "pbrtgpu_server_destroy": (None, [_P]),
    "pbrtgpu_server_submit_render": (C.c_int, [_P, _P, C.POINTER(PbrtCameraDesc), C.POINTER(PbrtSamplerDesc), _P,
                                               C.POINTER(C.c_uint64)]),
    "pbrtgpu_server_submit_query": (C.c_int, [_P, _P, _P, C.c_uint32, _P, _P, C.POINTER(C.c_uint64)]),
    "pbrtgpu_server_wait": (C.c_int, [_P, C.c_uint64, C.c_double, C.POINTER(C.c_int32)]),
    "pbrtgpu_server_drain": (C.c_int, [_P]),
    "pbrtgpu_server_stats": (C.c_int, [_P, C.POINTER(PbrtServerStats)]),
    "pbrtgpu_server_reset_stats": (C.c_int, [_P]),
}

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load the compiled library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(pbrt_rust_gb300 has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.pbrtgpu_abi_version() != ABI_VERSION:
        raise RuntimeError("pbrt_gpu ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


def get_trace_config() -> dict:
    lib = load()
    cfg = PbrtTraceConfig()
    check(lib.pbrtgpu_get_trace_config(C.byref(cfg)), lib)
    names = {v: k for k, v in TRACE_KERNELS.items()}
    return {"kernel": names[cfg.kernel], "refill": cfg.refill, "min_blocks": cfg.min_blocks,
            "render_kernel": names[cfg.render_kernel], "reorder": bool(cfg.reorder), "chunk": cfg.chunk}


def set_trace_config(kernel: str | None = None, refill: int | None = None, min_blocks: int | None = None,
                     render_kernel: str | None = None, reorder: bool | None = None,
                     chunk: int | None = None) -> None:
    """Choose the traversal kernels ('plain', 'pt', 'w4', 'w4pt') and their
    options; unset fields keep their current value."""
    lib = load()
    cur = get_trace_config()
    cfg = PbrtTraceConfig(TRACE_KERNELS[kernel or cur["kernel"]], refill or cur["refill"],
                          cur["min_blocks"] if min_blocks is None else min_blocks,
                          TRACE_KERNELS[render_kernel or cur["render_kernel"]],
                          int(cur["reorder"] if reorder is None else reorder),
                          cur["chunk"] if chunk is None else chunk)
    check(lib.pbrtgpu_set_trace_config(C.byref(cfg)), lib)


def set_trace_kernel(kernel: str, refill: int = 8) -> None:
    """Choose the kernel of pbrtgpu_intersect / intersect_p batches."""
    set_trace_config(kernel=kernel, refill=refill)


def get_trace_kernel() -> tuple[str, int]:
    c = get_trace_config()
    return c["kernel"], c["refill"]


def check(status: int, lib: C.CDLL | None = None) -> None:
    if status != PBRT_OK:
        lib = lib or load()
        msg = lib.pbrtgpu_last_error().decode(errors="replace")
        raise PbrtError(status, msg)


def f32p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def u32p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))
