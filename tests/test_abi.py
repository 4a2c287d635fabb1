"""The C-ABI library: it loads, exports every symbol the header declares, and
its host-side parts (argument checks, BVH build, status strings) work
without a GPU."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from pbrt_rust_gb300 import abi, generators as G
from pbrt_rust_gb300.gpu import GpuBVHAccel

HEADER = Path(__file__).resolve().parent.parent / "include" / "pbrt_gpu.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pbrtgpu_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_expected_surface():
    names = declared_functions()
    for must in ("pbrtgpu_bvh_create", "pbrtgpu_intersect", "pbrtgpu_intersect_p", "pbrtgpu_render",
                 "pbrtgpu_scene_create", "pbrtgpu_bvh_world_bound"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (pbrtgpu_[a-z0-9_]+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        assert n in abi.SIGNATURES, f"{n} has no ctypes signature"
        getattr(lib, n)


def test_status_strings(lib):
    assert lib.pbrtgpu_abi_version() == abi.ABI_VERSION == 2
    assert lib.pbrtgpu_status_str(0) == b"ok"
    assert lib.pbrtgpu_status_str(6) == b"traversal stack overflow"
    assert lib.pbrtgpu_status_str(999) == b"unknown status"


def test_invalid_arguments_fail_loudly(lib):
    h = C.c_void_p()
    assert lib.pbrtgpu_bvh_create(None, 3, 4, b"sah", C.byref(h)) == 1
    assert b"NULL" in lib.pbrtgpu_last_error()
    assert lib.pbrtgpu_intersect(None, None, 4, None, None) == 1
    with pytest.raises(ValueError):
        from pbrt_rust_gb300.scene import Shape
        from pbrt_rust_gb300.transform import Transform
        Shape.triangle_mesh(Transform(), None, False, [0, 1], np.zeros((3, 3)))


def test_streamed_walk_arguments_are_checked(lib):
    """pbrtgpu_intersect_streamed refuses a NULL handle, NULL rays or flags,
    both or neither output and a piece size outside 2^5..2^31 before it
    touches a device; a GPU-less host gets a status, never a CPU walk."""
    f = lib.pbrtgpu_intersect_streamed
    P = C.c_void_p
    buf = (C.c_uint32 * 64)()
    ptr = P(C.addressof(buf))
    assert f(None, ptr, 4, ptr, None, ptr, 16, None) == abi.PBRT_ERR_INVALID_ARGUMENT
    fake = P(1)  # never dereferenced: every check below fails first
    assert f(fake, None, 4, ptr, None, ptr, 16, None) == abi.PBRT_ERR_INVALID_ARGUMENT
    assert f(fake, ptr, 4, ptr, None, None, 16, None) == abi.PBRT_ERR_INVALID_ARGUMENT
    assert f(fake, ptr, 4, ptr, ptr, ptr, 16, None) == abi.PBRT_ERR_INVALID_ARGUMENT
    assert f(fake, ptr, 4, None, None, ptr, 16, None) == abi.PBRT_ERR_INVALID_ARGUMENT
    for shift in (0, 4, 32, 40):
        assert f(fake, ptr, 4, ptr, None, ptr, shift, None) == abi.PBRT_ERR_INVALID_ARGUMENT
    assert f(fake, ptr, 0, ptr, None, ptr, 16, None) == abi.PBRT_OK  # nothing to do


def test_bad_mesh_index_is_rejected(lib):
    d = abi.PbrtShapeDesc()
    pts = np.zeros(9, np.float32)
    idx = np.array([0, 1, 7], np.uint32)
    d.kind = abi.SHAPE_TRIANGLE_MESH
    d.object_to_world.m[:] = np.eye(4, dtype=np.float32).reshape(-1).tolist()
    d.object_to_world.m_inv[:] = np.eye(4, dtype=np.float32).reshape(-1).tolist()
    d.points = abi.f32p(pts)
    d.n_points = 3
    d.indices = abi.u32p(idx)
    d.n_indices = 3
    h = C.c_void_p()
    assert lib.pbrtgpu_bvh_create(C.byref(d), 1, 4, b"sah", C.byref(h)) == 1  # PBRT_ERR_INVALID_ARGUMENT
    assert b"out of range" in lib.pbrtgpu_last_error()


def test_host_build_matches_oracle_on_cpu(lib, oracle):
    """The product's BVH build (host side of pbrtgpu_bvh_create) equals the
    oracle's restatement of BVHAccelerator::new node for node."""
    prims, _ = G.ray_soup(3000, 1, seed=21)
    for sm in ("sah", "middle", "equal"):
        g = GpuBVHAccel(prims, 4, sm)
        o = oracle.OracleBVH(prims, 4, sm)
        assert np.array_equal(g.nodes().view(np.uint8), o.nodes().view(np.uint8))
        assert np.array_equal(g.primitive_order(), o.primitive_order())
        assert g.depth() == o.depth()


def test_no_cpu_fallback_without_a_gpu(lib):
    """Without a CUDA device the traversal fails with a status; it never
    computes on the CPU."""
    from conftest import HAS_GPU
    if HAS_GPU:
        pytest.skip("a GPU is present")
    prims, rays = G.ray_soup(100, 16, seed=2)
    g = GpuBVHAccel(prims)
    with pytest.raises(abi.PbrtError) as e:
        g.intersect(rays)
    assert e.value.status in (2, 10)


def test_render_task_range_is_checked(lib):
    """pbrtgpu_render_tasks rejects a range outside [0, num_tasks] before any
    device work."""
    from pbrt_rust_gb300.gpu import GpuSamplerRenderer, GpuScene
    prims, lights, cam, smp = G.c1_scene(res=16, n_spheres=2)
    scene = GpuScene(prims, lights)
    r = GpuSamplerRenderer(smp, cam, num_tasks=4)
    for lo, hi in ((3, 2), (0, 5)):
        with pytest.raises(abi.PbrtError) as e:
            r.render(scene, tasks=(lo, hi))
        assert e.value.status == 1 and b"task range" in lib.pbrtgpu_last_error()


def test_host_build_with_disks_and_cylinders_matches_oracle(lib, oracle):
    """Analytic shapes refine to one primitive each, with the bounds of
    disk.rs:68-74 / cylinder.rs:96-100, in the reference's BVH."""
    from pbrt_rust_gb300.scene import Primitive, Shape
    from pbrt_rust_gb300.transform import Transform
    prims, _ = G.ray_soup(200, 1, seed=4)
    for i in range(12):
        t = Transform.translate((i * 0.3 - 1.5, 0.2 * i, 0.1)) * Transform.rotate(30.0 * i, (1.0, 0.5, 0.0))
        s = (Shape.disk(t, None, False, 0.1 * i, 0.3, 0.05 * (i % 3), 360.0 - 20.0 * i) if i % 2
             else Shape.cylinder(t, None, i % 4 == 0, 0.2, -0.3, 0.1 * i, 360.0 - 25.0 * i))
        prims.append(Primitive.simple(s))
    g = GpuBVHAccel(prims, 4, "sah")
    o = oracle.OracleBVH(prims, 4, "sah")
    assert np.array_equal(g.nodes().view(np.uint8), o.nodes().view(np.uint8))
    assert np.array_equal(g.primitive_order(), o.primitive_order())
