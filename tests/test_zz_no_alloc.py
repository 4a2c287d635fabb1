"""pbrtgpu_render_noalloc - the render entry point that allocates nothing.

It exists for callers that cannot allocate device memory while rendering:
a serving process that reserves its device memory up front and admits work
against that fixed budget, or a frame loop that cannot afford the
device-wide synchronisation an allocation may cause.  Its scratch is one
fixed 64 MiB device array, so consecutive calls reuse whatever the previous
call left there; each call must still produce exactly the image the regular
entry point (pbrtgpu_render) produces.  This file is collected last and
builds everything it needs, so it passes alone in a fresh process as well as
after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from pbrt_rust_gb300 import abi, generators as G
from pbrt_rust_gb300.gpu import GpuSamplerRenderer, GpuScene
from pbrt_rust_gb300.scene import StratifiedSampler

pytestmark = pytest.mark.gpu
TOL = 1e-4  # the image tolerance of the render parity tests


def render_noalloc(lib, scene, renderer, out):
    """Calls the C-ABI entry point directly; `out` is a host array or a CUDA
    tensor of the film's shape."""
    ptr = C.c_void_p(out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data)
    return lib.pbrtgpu_render_noalloc(scene._h, C.byref(renderer._cam), C.byref(renderer._smp), ptr, None)


def test_noalloc_render_matches_render_on_consecutive_calls():
    lib = abi.load()
    prims, lights, cam, smp = G.c1_scene(res=96)
    scene = GpuScene(prims, lights)
    r = GpuSamplerRenderer(smp, cam)
    want = r.render(scene)
    assert want.max() > 0.1
    for _ in range(2):  # two calls in a row share the same scratch
        got = np.full_like(want, -1.0)
        st = render_noalloc(lib, scene, r, got)
        assert st == abi.PBRT_OK, lib.pbrtgpu_last_error()
        assert np.abs(got - want).max() <= TOL

    # a different frame right after: nothing left in the scratch may leak in
    r1 = GpuSamplerRenderer(StratifiedSampler.stratified(0, 96, 0, 96, 1, 1, True, 0.0, 1.0), cam)
    want1 = r1.render(scene)
    got1 = np.zeros_like(want1)
    assert render_noalloc(lib, scene, r1, got1) == abi.PBRT_OK, lib.pbrtgpu_last_error()
    assert np.abs(got1 - want1).max() <= TOL

    import torch
    dev = torch.full(want.shape, -1.0, dtype=torch.float32, device="cuda")
    assert render_noalloc(lib, scene, r, dev) == abi.PBRT_OK, lib.pbrtgpu_last_error()
    torch.cuda.synchronize()
    assert np.abs(dev.cpu().numpy() - want).max() <= TOL


def test_noalloc_refuses_frames_beyond_its_scratch():
    lib = abi.load()
    prims, lights, cam, _ = G.c1_scene(res=512)
    scene = GpuScene(prims, lights)
    big = GpuSamplerRenderer(StratifiedSampler.stratified(0, 512, 0, 512, 4, 4, True, 0.0, 1.0), cam)
    out = np.zeros((512, 512, 3), np.float32)
    assert render_noalloc(lib, scene, big, out) == 7  # PBRT_ERR_BUDGET
    assert b"bytes of scratch" in lib.pbrtgpu_last_error()
