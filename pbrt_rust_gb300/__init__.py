"""pbrt_rust_gb300: GB300-native BVH traversal, camera rays and direct
lighting for pbrt_rust scenes, behind the crate's aggregate/renderer
surface and a C ABI (include/pbrt_gpu.h)."""
from .abi import HIT_DTYPE, RAY_DTYPE, PbrtError, load
from .gpu import GpuBVHAccel, GpuSamplerRenderer, GpuScene
from .scene import (Camera, DiffuseAreaLight, Film, Filter, MatteMaterial, PointLight, Primitive, Shape,
                    StratifiedSampler, default_num_tasks, default_screen_window)
from .transform import Transform

__all__ = [
    "HIT_DTYPE", "RAY_DTYPE", "PbrtError", "load", "GpuBVHAccel", "GpuSamplerRenderer", "GpuScene", "Camera",
    "DiffuseAreaLight", "Film", "Filter", "MatteMaterial", "PointLight", "Primitive", "Shape",
    "StratifiedSampler", "default_num_tasks", "default_screen_window", "Transform",
]
