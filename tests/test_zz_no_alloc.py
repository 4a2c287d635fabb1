"""pbrtgpu_render_noalloc - the render entry point that allocates nothing.

It exists for callers that cannot allocate device memory while rendering:
a serving process that reserves its device memory up front and admits work
against that fixed budget, or a frame loop that cannot afford the
device-wide synchronisation an allocation may cause.  Its scratch is one
fixed 64 MiB device array, so consecutive calls reuse whatever the previous
call left there; each call must still produce exactly the image the regular
entry point (pbrtgpu_render) produces, bit for bit, and a call must leave
the device's free memory where it was.  This file is collected last and
builds everything it needs, so it passes alone in a fresh process as well as
after the other tests.
"""
import ctypes as C
import gc

import numpy as np
import pytest

from pbrt_rust_gb300 import abi, generators as G
from pbrt_rust_gb300.gpu import GpuSamplerRenderer, GpuScene
from pbrt_rust_gb300.scene import StratifiedSampler

pytestmark = pytest.mark.gpu


def render_noalloc(lib, scene, renderer, out):
    """Calls the C-ABI entry point directly; `out` is a host array or a CUDA
    tensor of the film's shape."""
    ptr = C.c_void_p(out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data)
    return lib.pbrtgpu_render_noalloc(scene._h, C.byref(renderer._cam), C.byref(renderer._smp), ptr, None)


def same_bits(a, b) -> bool:
    return a.shape == b.shape and np.array_equal(np.ascontiguousarray(a).view(np.uint32),
                                                 np.ascontiguousarray(b).view(np.uint32))


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
        assert same_bits(got, want)

    # a different frame right after: nothing left in the scratch may leak in
    r1 = GpuSamplerRenderer(StratifiedSampler.stratified(0, 96, 0, 96, 1, 1, True, 0.0, 1.0), cam)
    want1 = r1.render(scene)
    got1 = np.zeros_like(want1)
    assert render_noalloc(lib, scene, r1, got1) == abi.PBRT_OK, lib.pbrtgpu_last_error()
    assert same_bits(got1, want1)

    import torch
    dev = torch.full(want.shape, -1.0, dtype=torch.float32, device="cuda")
    assert render_noalloc(lib, scene, r, dev) == abi.PBRT_OK, lib.pbrtgpu_last_error()
    torch.cuda.synchronize()
    assert same_bits(dev.cpu().numpy(), want)


def test_noalloc_leaves_free_device_memory_unchanged():
    import torch
    lib = abi.load()
    prims, lights, cam, smp = G.c1_scene(res=80)
    scene = GpuScene(prims, lights)
    r4 = GpuSamplerRenderer(smp, cam)
    r1 = GpuSamplerRenderer(StratifiedSampler.stratified(0, 80, 0, 80, 1, 1, True, 0.0, 1.0), cam)
    out = np.zeros((80, 80, 3), np.float32)
    # the first call loads the render kernels' code, as any first launch does
    assert render_noalloc(lib, scene, r4, out) == abi.PBRT_OK, lib.pbrtgpu_last_error()
    gc.collect()
    gc.disable()  # no other object's device memory is released while measuring
    try:
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        for r in (r1, r4, r1):  # frames of other sizes reuse the same array
            assert render_noalloc(lib, scene, r, out) == abi.PBRT_OK, lib.pbrtgpu_last_error()
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
    finally:
        gc.enable()
    assert free1 == free0


def test_noalloc_refuses_frames_beyond_its_scratch():
    lib = abi.load()
    prims, lights, cam, _ = G.c1_scene(res=512)
    scene = GpuScene(prims, lights)
    big = GpuSamplerRenderer(StratifiedSampler.stratified(0, 512, 0, 512, 4, 4, True, 0.0, 1.0), cam)
    out = np.zeros((512, 512, 3), np.float32)
    assert render_noalloc(lib, scene, big, out) == 7  # PBRT_ERR_BUDGET
    assert b"bytes of scratch" in lib.pbrtgpu_last_error()
