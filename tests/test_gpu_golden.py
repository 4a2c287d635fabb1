"""The CUDA path against the committed golden fixtures (tests/golden/).

Same inputs as tests/test_golden.py, but the outputs come from the device
kernels through the C ABI: closest hits and any-hit bytes must equal the
stored values bit for bit, for every traversal kernel; the renders must
equal the stored images (bit for bit without spheres, within 1e-4 with
them, where CUDA's acosf/atan2f may round a sphere normal differently from
the host's libm).
"""
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import make_golden as MG  # noqa: E402

from pbrt_rust_gb300 import abi  # noqa: E402
from pbrt_rust_gb300.gpu import GpuBVHAccel, GpuSamplerRenderer, GpuScene  # noqa: E402
from pbrt_rust_gb300.scene import default_num_tasks  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(params=["plain", "pt", "w4", "w4pt", "w4spec"])
def kernel(request):
    before = abi.get_trace_config()
    abi.set_trace_config(kernel=request.param)
    yield request.param
    abi.set_trace_config(**before)


@pytest.mark.parametrize("name,scene", [("soup_closest.npz", lambda: MG.soup_inputs()[0]),
                                        ("spheres_closest.npz", lambda: MG.sphere_inputs()[0])])
def test_hits_equal_golden(kernel, name, scene):
    g = np.load(GOLDEN / name)
    bvh = GpuBVHAccel(scene(), 4, "sah")
    rays = MG.as_rays(g["rays"])
    assert np.array_equal(MG.hits_array(bvh.intersect(rays)), g["hits"])
    assert np.array_equal(bvh.intersect_p(rays), g["occluded"])


def test_renders_equal_golden():
    prims, lights, cam, smp = MG.sphere_inputs()[:4]
    img = GpuSamplerRenderer(smp, cam, num_tasks=default_num_tasks(48, 48)).render(GpuScene(prims, lights))
    want = np.load(GOLDEN / "render_c1_48.npz")["rgb"]
    assert np.abs(img - want).max() <= TOL and want.max() > 0.1

    prims, lights, cam, smp = MG.tris_inputs()
    img = GpuSamplerRenderer(smp, cam, num_tasks=default_num_tasks(40, 40)).render(GpuScene(prims, lights))
    assert np.array_equal(img.view(np.uint32), np.load(GOLDEN / "render_tris_40.npz")["rgb"].view(np.uint32))
