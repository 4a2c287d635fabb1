"""Standalone workloads for profilers (ncu) and quick timing.

  python -m pbrt_rust_gb300.profile trace  [--rays N] [--any] [--host-out] [--repeat R]
  python -m pbrt_rust_gb300.profile render [--res R] [--spp-side S] [--repeat R]
  python -m pbrt_rust_gb300.profile batch  [--scenes N] [--repeat R]
  python -m pbrt_rust_gb300.profile served [--scenes N] [--requests Q] [--slots K] [--repeat R]

`trace` and `render` use the 708x708 heightfield scene; `trace` runs R
closest-hit (or any-hit) passes over N incoherent rays (with --host-out the
closest hits go to pinned host memory: the walk that writes them out chunk
by chunk), `render` R frames of
the direct-lighting wavefront.  `batch` renders the multi-scene workload
(N scenes of 1k-256k triangles + 0-32 spheres, 128-512 squared, 1/4/16 spp)
as one batch R times, with the tuning the autotuner picks for it (binary
walks, 256 threads, refill 32: the flat traversal stages).  Each pass is
timed with CUDA events on its stream.  `served` builds the serving workload
(N resident scenes of 10k-1M triangles, Q requests: renders 128-512 squared
at 1/4 spp and ray batches of 2^14-2^18 rays), runs every request once
through the one-request calls, then R floods of all Q through a server with
K slots, and prints wall-clock requests/s of both.
"""
from __future__ import annotations

import argparse
import ctypes as C
import sys
import time

import numpy as np


def serving_pool(n_scenes: int = 32, threads: int = 8):
    """The resident scenes of the serving workload: n_scenes random-triangle
    soups of 10k-1M triangles (log uniform) with 0-32 spheres, two lights
    each.  Returns [(GpuScene, GpuBVHAccel, Camera)]."""
    from concurrent.futures import ThreadPoolExecutor

    from . import generators as G
    from .gpu import GpuScene

    def one(i):
        prims, lights, cam, _ = G.multi_scene(i, seed=G.config_seed(4, i), tri_range=(10000, 1000000),
                                              res_choices=(128,), spp_choices=(1,))
        sc = GpuScene(prims, lights)
        return sc, sc.aggregate(), cam

    with ThreadPoolExecutor(threads) as ex:  # host BVH builds release the GIL
        return list(ex.map(one, range(n_scenes)))


def serving_requests(pool, n_requests: int, device, seed: int | None = None):
    """The request stream over `pool`: ("render", scene, renderer, out) or
    ("query", bvh, rays, out) tuples, rays and outputs on `device`; every
    ray batch has its own rays."""
    import torch

    from . import generators as G
    from .gpu import GpuSamplerRenderer
    from .scene import Camera, Film, Filter, StratifiedSampler
    reqs = []
    for spec in G.serving_requests(n_requests, len(pool), seed=seed):
        sc, bvh, cam = pool[spec["scene"]]
        if spec["kind"] == "render":
            res, side = spec["res"], 1 if spec["spp"] == 1 else 2
            film = Film.image(res, res, Filter.mean(0.5, 0.5))
            c = G.orbit_camera(Camera.perspective(cam.camera_to_world, cam.screen_window, 0.0, 1.0, 0.0, 1e30, 60.0,
                                                  film), spec["radius"], spec["azimuth"])
            smp = StratifiedSampler.stratified(0, res, 0, res, side, side, True, 0.0, 1.0)
            reqs.append(("render", sc, GpuSamplerRenderer(smp, c), torch.empty((res, res, 3), device=device)))
        else:
            lo, hi = bvh.world_bound()
            rays = G.incoherent_rays(G.PCG32(spec["seed"]), spec["n"], lo, hi)
            rd = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(device)
            reqs.append(("query", bvh, rd, torch.empty((spec["n"], 4), device=device)))
    return reqs


def run_plain(reqs, stream, arrivals=None) -> list:
    """Every request through its one-request call, each finished before the
    next starts (renders return after the frame; queries synchronise); with
    `arrivals` (seconds from the start) a request starts no earlier than its
    arrival.  Returns each request's latency in seconds: completion minus
    arrival (minus its own start without arrivals)."""
    lat = []
    t0 = time.perf_counter()
    for k, r in enumerate(reqs):
        if arrivals is not None:
            while time.perf_counter() - t0 < arrivals[k]:
                pass
            start = t0 + arrivals[k]
        else:
            start = time.perf_counter()
        if r[0] == "render":
            r[2].render(r[1], out=r[3], stream=stream)
        else:
            r[1].intersect(r[2], out=r[3], stream=stream)
            stream.synchronize()
        lat.append(time.perf_counter() - start)
    return lat


def run_served(srv, reqs, outs, arrivals=None) -> dict:
    """Submits every request (at `arrivals` seconds from the start when
    given, else at once), waits for all, returns the server's statistics."""
    srv.reset_stats()
    tickets = []
    t0 = time.perf_counter()
    for k, (r, o) in enumerate(zip(reqs, outs)):
        if arrivals is not None:
            while time.perf_counter() - t0 < arrivals[k]:
                pass
        tickets.append(srv.submit_render(r[1], r[2], out=o) if r[0] == "render"
                       else srv.submit_query(r[1], r[2], out=o))
    for t in tickets:
        srv.wait(t)
    return srv.stats()


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["trace", "render", "batch", "served"])
    ap.add_argument("--scenes", type=int, default=64)
    ap.add_argument("--rays", type=int, default=1 << 20)
    ap.add_argument("--any", action="store_true")
    ap.add_argument("--host-out", action="store_true", help="trace: closest hits into pinned host memory")
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--res", type=int, default=256)
    ap.add_argument("--spp-side", type=int, default=2)
    ap.add_argument("--requests", type=int, default=400)
    ap.add_argument("--slots", type=int, default=2)
    ap.add_argument("--tuning", default="", help="served: batch tuning as key=value,... (GpuServer tuning)")
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
    if a.what == "served":
        from .server import GpuServer
        pool = serving_pool(min(a.scenes, 32))
        reqs = serving_requests(pool, a.requests, torch.device("cuda"))
        run_plain(reqs[:20], stream)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run_plain(reqs, stream)
        plain_s = time.perf_counter() - t0
        tuning = {k: (v if k.endswith("kernel") else int(v))
                  for k, v in (kv.split("=") for kv in a.tuning.split(",") if kv)}
        srv = GpuServer(slots=a.slots, tuning=tuning or None, max_jobs=256, max_samples=1 << 24,
                        max_film_pixels=1 << 22, max_query_rays=1 << 20, max_tasks=1 << 14)
        outs = [torch.empty_like(r[3]) for r in reqs]
        for _ in range(a.repeat):
            st = run_served(srv, reqs, outs)
            print(f"served: {st['requests_per_s']:.0f} requests/s, {st['batches']} batches, mean "
                  f"{st['mean_batch_requests']:.1f} requests, p50 {st['p50_ms']:.2f} ms, p99 {st['p99_ms']:.2f} ms")
        srv.close()
        print(f"plain: {len(reqs) / plain_s:.0f} requests/s")
        return 0
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
                          device="cpu" if a.host_out and not a.any else "cuda")
        if a.host_out and not a.any:
            out = out.pin_memory()
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
