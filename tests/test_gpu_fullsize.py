"""Parity at the benchmark's own sizes: the 708x708-vertex heightfield
(999,698 triangles + the 2-triangle light) with its 2^22 incoherent rays,
and its 1024x1024 16-spp direct-lighting frame, against the oracle.

Triangle-only scenes are exact IEEE f32 end to end, so hits and images are
compared bit for bit."""
import numpy as np
import pytest

from pbrt_rust_gb300 import abi, generators as G
from pbrt_rust_gb300.gpu import GpuBVHAccel, GpuSamplerRenderer, GpuScene
from pbrt_rust_gb300.scene import SceneDescription, default_num_tasks

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def heightfield():
    prims, lights, cam, smp, rays = G.heightfield(n_rays=1 << 22)
    return prims, lights, cam, smp, rays


@pytest.mark.parametrize("name", ["w4pt", "plain", "packet"])
def test_heightfield_rays_match_oracle(oracle, heightfield, name):
    prims, _, _, _, rays = heightfield
    before = abi.get_trace_config()
    abi.set_trace_config(kernel=name)
    try:
        g, o = GpuBVHAccel(prims, 4, "sah"), oracle.OracleBVH(prims, 4, "sah")
        want = o.intersect(rays)
        assert (want["prim"] >= 0).sum() > len(rays) // 4
        assert np.array_equal(g.intersect(rays).view(np.uint32), want.view(np.uint32))
        assert np.array_equal(g.intersect_p(rays), o.intersect_p(rays))
    finally:
        abi.set_trace_config(**before)


@pytest.fixture(scope="module")
def heightfield_frame(oracle, heightfield):
    prims, lights, cam, smp, _ = heightfield
    nt = default_num_tasks(cam.film.x_res, cam.film.y_res)
    return oracle.render(SceneDescription(prims, lights, 4, "sah"), cam, smp, nt)


@pytest.mark.parametrize("render_kernel", ["plain", "packet", "w4"])
def test_heightfield_frame_matches_oracle(heightfield, heightfield_frame, render_kernel):
    prims, lights, cam, smp, _ = heightfield
    nt = default_num_tasks(cam.film.x_res, cam.film.y_res)
    before = abi.get_trace_config()
    abi.set_trace_config(render_kernel=render_kernel)
    try:
        gpu = GpuSamplerRenderer(smp, cam, num_tasks=nt).render(GpuScene(prims, lights, 4, "sah"))
    finally:
        abi.set_trace_config(**before)
    ref = heightfield_frame
    assert gpu.shape == (1024, 1024, 3) and ref.max() > 0.1
    assert np.array_equal(gpu.view(np.uint32), ref.view(np.uint32))
