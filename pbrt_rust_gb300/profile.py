"""Standalone workloads for profilers (ncu) and quick timing.

  python -m pbrt_rust_gb300.profile trace  [--rays N] [--any] [--repeat R]
  python -m pbrt_rust_gb300.profile render [--res R] [--spp-side S] [--repeat R]
  python -m pbrt_rust_gb300.profile batch  [--scenes N] [--repeat R]

`trace` and `render` use the 708x708 heightfield scene; `trace` runs R
closest-hit (or any-hit) passes over N incoherent rays, `render` R frames of
the direct-lighting wavefront.  `batch` renders the multi-scene workload
(N scenes of 1k-256k triangles + 0-32 spheres, 128-512 squared, 1/4/16 spp)
as one batch R times, with the tuning the autotuner picks for it (binary
walks, 256 threads, refill 32: the flat traversal stages).  Each pass is
timed with CUDA events on its stream.
"""
from __future__ import annotations

import argparse
import ctypes as C
import sys

import numpy as np


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["trace", "render", "batch"])
    ap.add_argument("--scenes", type=int, default=64)
    ap.add_argument("--rays", type=int, default=1 << 20)
    ap.add_argument("--any", action="store_true")
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--res", type=int, default=256)
    ap.add_argument("--spp-side", type=int, default=2)
    a = ap.parse_args(argv)
    import torch

    from . import abi, generators as G
    from .gpu import GpuBVHAccel, GpuSamplerRenderer, GpuScene
    from .scene import StratifiedSampler

    lib = abi.load()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    times = []
    if a.what == "batch":
        from concurrent.futures import ThreadPoolExecutor

        from .batch import GpuBatch

        def one(i):
            p, li, c, sm = G.multi_scene(i)
            return GpuScene(p, li), GpuSamplerRenderer(sm, c)

        with ThreadPoolExecutor(8) as ex:  # host BVH builds release the GIL
            items = list(ex.map(one, range(a.scenes)))
        px = [r.camera.film.x_res * r.camera.film.y_res for _, r in items]
        samples = sum(n * r.sampler.x_samples * r.sampler.y_samples for n, (_, r) in zip(px, items))
        b = GpuBatch(max_jobs=a.scenes, max_tasks=64 * a.scenes, max_samples=samples,
                     max_light_samples=2 * samples, max_film_pixels=sum(px))
        b.set_tuning(extend_kernel="pair", shadow_kernel="pair", block=256, chunk=64, refill=32, refill_shadow=32,
                     use_graph=1)
        outs = [torch.empty((r.camera.film.y_res, r.camera.film.x_res, 3), device="cuda") for _, r in items]
        for _ in range(a.repeat):
            for (sc, r), o in zip(items, outs):
                b.add_render(sc, r, out=o)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            b.launch(stream)
            e1.record(stream)
            b.wait()
            times.append(e0.elapsed_time(e1))
        print(f"batch: {' '.join(f'{t:.3f}' for t in times)} ms; best {a.scenes / (min(times) / 1e3):.0f} renders/s")
        return 0
    prims, lights, cam, smp, rays = G.heightfield(n_rays=a.rays if a.what == "trace" else 0)
    if a.what == "trace":
        bvh = GpuBVHAccel(prims, 4, "sah")
        rd = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
        out = torch.empty((a.rays, 4) if not a.any else (a.rays,), dtype=torch.float32 if not a.any else torch.uint8,
                          device="cuda")
        fn = lib.pbrtgpu_intersect_p if a.any else lib.pbrtgpu_intersect
        for _ in range(a.repeat):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            abi.check(fn(bvh._h, C.c_void_p(rd.data_ptr()), a.rays, C.c_void_p(out.data_ptr()), sh), lib)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        unit = a.rays
    else:
        from .scene import Camera, Film, Filter
        film = Film.image(a.res, a.res, Filter.mean(0.5, 0.5))
        cam = Camera.perspective(cam.camera_to_world, cam.screen_window, 0.0, 1.0, 0.0, 1e30, cam.fov, film)
        smp = StratifiedSampler.stratified(0, a.res, 0, a.res, a.spp_side, a.spp_side, True, 0.0, 1.0)
        scene = GpuScene(prims, lights)
        r = GpuSamplerRenderer(smp, cam)
        img = torch.empty((a.res, a.res, 3), dtype=torch.float32, device="cuda")
        for _ in range(a.repeat):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r.render(scene, out=img, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        unit = a.res * a.res * a.spp_side * a.spp_side
    print(f"{a.what}: {' '.join(f'{t:.3f}' for t in times)} ms; best {unit / (min(times) / 1e3) / 1e6:.1f} M/s")
    return 0


if __name__ == "__main__":
    sys.exit(main())
