"""Benchmark: closest-hit rays/s on the 1M-triangle heightfield.

Workload (the configuration the headline metric is quoted on): a
708x708-vertex heightfield (999,698 triangles) plus its 2-triangle area
light, SAH BVH built with the reference's algorithm, and 2^22 incoherent
rays (origins uniform in the mesh bounds inflated by 1, directions uniform
on the sphere).  One step = one closest-hit pass over all 2^22 rays.

  value       device-resident rays/hits, kernel time from CUDA events on
              the launching stream; L2 flushed (256 MiB write) between steps
  e2e         the same pass through the C ABI with pinned HOST buffers and
              the synchronisation inside the timed step: the traversal reads
              the rays from and writes the hits to the mapped host memory
              (Grace memory over NVLink-C2C); `e2e.staged` is the same call
              with PBRT_HOST_MAPPED=0, i.e. host->device copies of the rays,
              traversal and device->host copies of the hits pipelined in
              four pieces
  roofline    algorithmic bytes per launch (32 B per node tested + 48 B per
              triangle tested + 32 B ray + 16 B hit, counted by the oracle's
              reference-order traversal on a 2^16-ray sample and scaled)
              over the measured launch time, against the measured HBM copy
              bandwidth
  cpu_baseline  the CPU oracle (a C++ restatement of the reference's
              BVHAccelerator::intersect): whole passes over the same rays for
              at least 10 s, all host threads

--impl reference times that CPU implementation alone on the same workload.
Under torchrun each rank traces its own 2^22 rays against a replicated BVH
(no collective in the data path); value = all ranks' rays / max rank time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GPU Mrays/s (1M tris) & p50/p99 render latency vs plain kernel at equal RMSE"
WORKLOAD = "heightfield-708x708 (999,700 tris, SAH BVH) + 2^22 incoherent rays, closest hit"
N_RAYS = 1 << 22
HBM_FALLBACK_GBS = 6800.0
REASON_BITS = {
    0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap", 0x8: "hw_slowdown",
    0x10: "sync_boost", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown",
    0x100: "display_clock_setting",
}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return HBM_FALLBACK_GBS, "fallback"


def committed_traffic():
    """dram__bytes_read.sum + dram__bytes_write.sum of one closest-hit launch
    on this workload, from the committed ncu summary (None without one)."""
    p = ROOT / "profiles" / "k_trace4_persistent_heightfield_4M_rays.md"
    if p.exists():
        m = re.search(r"^dram_bytes_per_launch = (\d+)$", p.read_text(), re.M)
        if m:
            return {"dram_bytes_per_launch": int(m.group(1)), "source": str(p.relative_to(ROOT))}
    return None


class ClockSampler:
    """nvidia-smi samples of SM clocks and throttle reasons while running."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = "clocks.sm,clocks.max.sm,clocks_event_reasons.active"
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def wait_first(self, timeout: float):
        t0 = time.perf_counter()
        while self.proc and not self.samples and time.perf_counter() - t0 < timeout:
            time.sleep(0.02)

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 3:
                try:
                    self.samples.append((float(parts[0]), float(parts[1]), int(parts[2], 16)))
                except ValueError:
                    pass

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [s[0] for s in self.samples]
        mx = max(s[1] for s in self.samples)
        bits = 0
        for s in self.samples:
            bits |= s[2]
        reasons = [name for b, name in REASON_BITS.items() if bits & b and b != 0x1]
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def build_workload(n_rays: int):
    from pbrt_rust_gb300 import generators as G
    prims, lights, cam, smp, rays = G.heightfield(n_rays=n_rays)
    return prims, lights, cam, smp, rays


def cpu_baseline_leg(prims, rays, nthreads: int, min_seconds: float = 10.0, sample: int = 1 << 16):
    """The CPU-baseline leg, the only part of the GPU arm that runs the oracle:
    whole passes over `rays` on the host until `min_seconds` have passed, and
    the algorithmic bytes per ray of the roofline - 32 B per node tested +
    48 B per triangle tested + 32 B ray + 16 B hit, the tests counted by the
    oracle's reference-order traversal of a 2^16-ray sample.
    Returns (rays/s, seconds, passes, (bytes/ray, nodes/ray, triangles/ray))."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    ob = O.OracleBVH(prims, 4, "sah")
    rays = np.ascontiguousarray(rays)
    ob.intersect(rays[:1024], nthreads=nthreads)
    passes, t0 = 0, time.perf_counter()
    while True:
        ob.intersect(rays, nthreads=nthreads)
        passes += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            break
    sub = np.ascontiguousarray(rays[:: max(1, len(rays) // sample)][:sample])
    _, cnt = ob.intersect(sub, counters=True)
    nodes, tris = cnt[0] / len(sub), cnt[1] / len(sub)
    return passes * len(rays) / dt, dt, passes, (32.0 * nodes + 48.0 * tris + 32.0 + 16.0, nodes, tris)


def build_multi_scene(n: int, threads: int = 8):
    """The batched multi-scene workload: n scenes of 1k-256k triangles (log
    uniform) + 0-32 spheres, 128/256/512 squared at 1/4/16 spp."""
    from concurrent.futures import ThreadPoolExecutor

    from pbrt_rust_gb300 import generators as G
    from pbrt_rust_gb300.gpu import GpuSamplerRenderer, GpuScene

    def one(i):
        prims, lights, cam, smp = G.multi_scene(i)
        return GpuScene(prims, lights), GpuSamplerRenderer(smp, cam)

    with ThreadPoolExecutor(threads) as ex:  # host BVH builds release the GIL
        return list(ex.map(one, range(n)))


def bench_batched(torch, dev, stream, n_scenes: int = 64):
    """Renders/s of n_scenes renders: one pbrtgpu_render per scene in turn
    (the plain one-scene-per-launch path) against one autotuned batch."""
    from pbrt_rust_gb300.batch import GpuBatch
    items = build_multi_scene(n_scenes)
    outs = [torch.empty((r.camera.film.y_res, r.camera.film.x_res, 3), device=dev) for _, r in items]
    samples = sum(r.camera.film.x_res * r.camera.film.y_res * r.sampler.x_samples * r.sampler.y_samples
                  for _, r in items)
    film = sum(r.camera.film.x_res * r.camera.film.y_res for _, r in items)
    for (sc, r), o in zip(items, outs):  # warm-up: uploads, scratch
        r.render(sc, out=o, stream=stream)
    torch.cuda.synchronize(dev)
    reps = 2
    t0 = time.perf_counter()
    for _ in range(reps):
        for (sc, r), o in zip(items, outs):
            r.render(sc, out=o, stream=stream)
    torch.cuda.synchronize(dev)
    plain_s = (time.perf_counter() - t0) / reps
    ref = [o.clone() for o in outs]
    b = GpuBatch(max_jobs=n_scenes, max_tasks=64 * n_scenes, max_samples=samples, max_light_samples=2 * samples,
                 max_film_pixels=film)
    bouts = [torch.empty_like(o) for o in outs]
    for (sc, r), o in zip(items, bouts):
        b.add_render(sc, r, out=o)
    tuned, tuned_ms = b.autotune(stream=stream, repeats=2)
    b.wait()
    times = []
    for _ in range(3):
        for (sc, r), o in zip(items, bouts):
            b.add_render(sc, r, out=o)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        b.launch(stream)
        b.wait()
        times.append(time.perf_counter() - t0)
    stats = b.stats()
    exact = all(torch.equal(a.view(torch.int32), c.view(torch.int32)) for a, c in zip(bouts, ref))
    if not exact:
        raise RuntimeError("batched renders differ from the one-scene renders")
    batch_s = statistics.median(times)
    return {"scenes": n_scenes, "samples": samples, "plain_renders_per_s": n_scenes / plain_s,
            "batched_renders_per_s": n_scenes / batch_s, "speedup": plain_s / batch_s,
            "batched_ms": 1e3 * batch_s, "plain_ms": 1e3 * plain_s, "autotuned": tuned,
            "kernels_per_launch": stats["kernels"], "graph": bool(stats["graph"]), "bit_exact": exact}


def bench_served(torch, dev, stream, n_scenes: int = 32, n_requests: int = 400, rate: float = 1000.0):
    """Requests/s and latency of the serving loop against the plain path
    (one request at a time through pbrtgpu_render / pbrtgpu_intersect) on
    the same request stream; all outputs device-resident."""
    from concurrent.futures import ThreadPoolExecutor

    from pbrt_rust_gb300 import generators as G
    from pbrt_rust_gb300.gpu import GpuSamplerRenderer, GpuScene
    from pbrt_rust_gb300.scene import Camera, Film, Filter, StratifiedSampler
    from pbrt_rust_gb300.server import GpuServer

    def one(i):
        prims, lights, cam, smp = G.multi_scene(i, seed=G.config_seed(4, i), tri_range=(10000, 1000000),
                                                res_choices=(128,), spp_choices=(1,))
        sc = GpuScene(prims, lights)
        return sc, sc.aggregate(), cam

    with ThreadPoolExecutor(8) as ex:
        pool = list(ex.map(one, range(n_scenes)))
    reqs = []
    for spec in G.serving_requests(n_requests, n_scenes):
        sc, bvh, cam = pool[spec["scene"]]
        if spec["kind"] == "render":
            res, side = spec["res"], 1 if spec["spp"] == 1 else 2
            film = Film.image(res, res, Filter.mean(0.5, 0.5))
            c = G.orbit_camera(Camera.perspective(cam.camera_to_world, cam.screen_window, 0.0, 1.0, 0.0, 1e30, 60.0,
                                                  film), spec["radius"], spec["azimuth"])
            smp = StratifiedSampler.stratified(0, res, 0, res, side, side, True, 0.0, 1.0)
            reqs.append(("render", sc, GpuSamplerRenderer(smp, c), torch.empty((res, res, 3), device=dev)))
        else:
            lo, hi = bvh.world_bound()
            rays = G.incoherent_rays(G.PCG32(spec["seed"]), spec["n"], lo, hi)
            rd = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
            reqs.append(("query", bvh, rd, torch.empty((spec["n"], 4), device=dev)))

    def plain(r):
        if r[0] == "render":
            r[2].render(r[1], out=r[3], stream=stream)  # returns after the frame is done
        else:
            r[1].intersect(r[2], out=r[3], stream=stream)
            stream.synchronize()

    for r in reqs[:20]:
        plain(r)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for r in reqs:
        plain(r)
    plain_s = time.perf_counter() - t0
    ref = [r[3].clone() for r in reqs]
    srv = GpuServer(slots=2, max_jobs=256, max_samples=1 << 24, max_film_pixels=1 << 22, max_query_rays=1 << 20,
                    max_tasks=1 << 14)
    outs = [torch.empty_like(r[3]) for r in reqs]

    def serve(arrivals=None):
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

    serve()
    flood = serve()
    torch.cuda.synchronize(dev)
    exact = all(torch.equal(a.view(torch.int32), b.view(torch.int32)) for a, b in zip(outs, ref))
    if not exact:
        raise RuntimeError("served results differ from the one-request results")
    poisson = serve(G.poisson_arrivals(len(reqs), rate, seed=9))
    srv.close()
    n_render = sum(1 for r in reqs if r[0] == "render")
    return {"scenes": n_scenes, "requests": len(reqs), "renders": n_render, "queries": len(reqs) - n_render,
            "plain_requests_per_s": len(reqs) / plain_s, "served_requests_per_s": flood["requests_per_s"],
            "speedup": flood["requests_per_s"] * plain_s / len(reqs),
            "flood_p50_ms": flood["p50_ms"], "flood_p99_ms": flood["p99_ms"],
            "flood_mean_batch": flood["mean_batch_requests"],
            "poisson_rate": rate, "poisson_requests_per_s": poisson["requests_per_s"],
            "poisson_p50_ms": poisson["p50_ms"], "poisson_p99_ms": poisson["p99_ms"],
            "poisson_mean_batch": poisson["mean_batch_requests"], "bit_exact": exact}


def bench_rmse(torch, dev, stream):
    """The plain render config (512x512, 2x2 strata, ground, 64 spheres,
    point + area light): frame time and RMSE (linear RGB) against the same
    scene at 8x8 strata (64 spp, the most a pixel takes; same task split, so
    the same task seams), whose own noise adds about 3 % to the figure.  The
    batched and served forms produce bit-identical images, hence the same
    RMSE."""
    from pbrt_rust_gb300 import generators as G
    from pbrt_rust_gb300.gpu import GpuSamplerRenderer, GpuScene
    prims, lights, cam, smp = G.c1_scene(res=512)
    scene = GpuScene(prims, lights)
    img = torch.empty((512, 512, 3), dtype=torch.float32, device=dev)
    r4 = GpuSamplerRenderer(smp, cam)
    r4.render(scene, out=img, stream=stream)
    t = []
    for _ in range(5):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        r4.render(scene, out=img, stream=stream)
        t.append(time.perf_counter() - t0)
    _, _, _, smp64 = G.c1_scene(res=512, spp_side=8)
    ref = torch.empty_like(img)
    GpuSamplerRenderer(smp64, cam).render(scene, out=ref, stream=stream)
    torch.cuda.synchronize(dev)
    rmse = float(torch.sqrt(torch.mean((img - ref) ** 2)).item())
    return {"ms_mean": 1e3 * statistics.mean(t), "ms_min": 1e3 * min(t), "spp": 4, "rmse_vs_64spp": rmse,
            "reference_mean": float(ref.mean().item())}


def bench_instanced(torch, dev, stream, n_instances: int = 256, tris_per_tree: int = 20000,
                    n_rays: int = 1 << 22):
    """TransformedPrimitive instancing: the instanced forest against the
    same forest with every instance copied out, closest hit of 2^22 rays
    aimed into the forest (device-resident rays, CUDA events, L2 flushed)."""
    from pbrt_rust_gb300 import abi, generators as G
    from pbrt_rust_gb300.gpu import GpuBVHAccel
    lib = abi.load()
    prims, _, _, _, flat = G.instanced_forest(n_instances=n_instances, tris_per_tree=tris_per_tree, seed=1)
    rays = G.rays_toward_center(G.PCG32(77), n_rays, radius=14.0, target=4.0)
    inst = GpuBVHAccel(prims, 4, "sah", build_on_device=True)
    copied = GpuBVHAccel(flat, 4, "sah", build_on_device=True)
    sh = C.c_void_p(stream.cuda_stream)
    rays_dev = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    out = {}
    hits = {}
    for name, b in (("instanced", inst), ("copied_out", copied)):
        h = torch.empty((n_rays, 4), dtype=torch.float32, device=dev)
        rp, hp = C.c_void_p(rays_dev.data_ptr()), C.c_void_p(h.data_ptr())
        ms = []
        with torch.cuda.stream(stream):
            for k in range(8):
                flush.zero_()
                a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                abi.check(lib.pbrtgpu_intersect(b._h, rp, n_rays, hp, sh), lib)
                e.record(stream)
                if k >= 3:
                    ms.append((a, e))
        torch.cuda.synchronize(dev)
        t = statistics.mean(a.elapsed_time(e) for a, e in ms)
        out[name] = {"mrays_s": n_rays / t / 1e3, "ms": t, "device_bytes": b.device_bytes(),
                     "primitives": b.num_primitives(), "nodes": b.num_nodes()}
        hits[name] = h
    agree = (hits["instanced"][:, 0].view(torch.int32) == hits["copied_out"][:, 0].view(torch.int32))
    out.update({"instances": n_instances, "tris_per_tree": tris_per_tree,
                "copied_out_triangles": sum(p.shape.num_primitives() for p in flat),
                "same_hit_fraction": float(agree.float().mean().item()),
                "memory_ratio": out["copied_out"]["device_bytes"] / out["instanced"]["device_bytes"],
                "what": "forest of tree/post definitions placed by rotated, scaled instances; closest hit of "
                        "2^22 rays aimed into it; hit ids of the two scenes agree up to f32 rounding"})
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    prims, _, _, _, rays = build_workload(N_RAYS)
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    ob = O.OracleBVH(prims, 4, "sah")
    # one step = the whole 2^22-ray pass, as on the GPU (about 0.3 s on 16 cores)
    per_step = N_RAYS
    rays = np.ascontiguousarray(rays)
    for _ in range(args.warmup):
        ob.intersect(rays, nthreads=nthreads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ob.intersect(rays, nthreads=nthreads)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = per_step / (ms / 1e3) / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD, "sample": f"{per_step} rays per step", "threads": nthreads},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": nthreads, "kind": "port",
                         "sample": f"all 2^22 rays per step, {args.steps} steps"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())
    from pbrt_rust_gb300 import abi
    from pbrt_rust_gb300.gpu import GpuBVHAccel, GpuSamplerRenderer, GpuScene

    lib = abi.load()
    prims, lights, cam, smp, rays = build_workload(N_RAYS)
    t0 = time.perf_counter()
    bvh = GpuBVHAccel(prims, 4, "sah")
    build_s = time.perf_counter() - t0
    # the same BVH built by the device kernels (PBRT_BUILD_ON_DEVICE)
    GpuBVHAccel(prims[:1], 4, "sah", build_on_device=True)  # warm-up: context, kernel loading
    t0 = time.perf_counter()
    dbvh = GpuBVHAccel(prims, 4, "sah", build_on_device=True)
    dbuild_s = time.perf_counter() - t0
    same_tree = (np.array_equal(dbvh.nodes().view(np.uint8), bvh.nodes().view(np.uint8))
                 and np.array_equal(dbvh.primitive_order(), bvh.primitive_order()))
    del dbvh
    stream = torch.cuda.Stream(device=dev)
    sh = C.c_void_p(stream.cuda_stream)
    rays_dev = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
    hits_dev = torch.empty((N_RAYS, 4), dtype=torch.float32, device=dev)
    occ_dev = torch.empty((N_RAYS,), dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    rp, hp, op = C.c_void_p(rays_dev.data_ptr()), C.c_void_p(hits_dev.data_ptr()), C.c_void_p(occ_dev.data_ptr())

    def closest():
        abi.check(lib.pbrtgpu_intersect(bvh._h, rp, N_RAYS, hp, sh), lib)

    def anyhit():
        abi.check(lib.pbrtgpu_intersect_p(bvh._h, rp, N_RAYS, op, sh), lib)

    def timed(fn, steps, warmup):
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                flush.zero_()
                fn()
        torch.cuda.synchronize(dev)
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        evs = []
        with torch.cuda.stream(stream):
            for _ in range(steps):
                flush.zero_()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                evs.append((a, b))
        torch.cuda.synchronize(dev)
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        return [a.elapsed_time(b) for a, b in evs]

    # nvidia-smi samples every 100 ms; the sampler runs across every timed
    # region below (closest, any hit, e2e, render), and the closest-hit loop
    # starts only once the first sample has arrived
    clk = ClockSampler(torch.cuda.current_device()).__enter__()
    clk.wait_first(5.0)
    ms_closest = timed(closest, args.steps, args.warmup)
    ms_any = timed(anyhit, max(3, args.steps // 2), args.warmup)

    print(f"[bench] closest {statistics.mean(ms_closest):.3f} ms/step, any {statistics.mean(ms_any):.3f} ms/step",
          file=sys.stderr, flush=True)
    # e2e: pinned host buffers through the C ABI, read and written in place
    # (default) or staged through device copies (PBRT_HOST_MAPPED=0)
    rays_host = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
    hits_host = torch.empty((N_RAYS, 4), dtype=torch.float32).pin_memory()
    rh, hh = C.c_void_p(rays_host.data_ptr()), C.c_void_p(hits_host.data_ptr())
    torch.cuda.synchronize(dev)
    hits_want = hits_dev.cpu().view(torch.int32)

    def e2e_pass(mapped: bool) -> float:
        os.environ["PBRT_HOST_MAPPED"] = "1" if mapped else "0"
        for _ in range(args.warmup):
            abi.check(lib.pbrtgpu_intersect(bvh._h, rh, N_RAYS, hh, sh), lib)
        t = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            abi.check(lib.pbrtgpu_intersect(bvh._h, rh, N_RAYS, hh, sh), lib)
            t.append(time.perf_counter() - t0)
        # the host copy of the result must equal the device-resident one
        if not torch.equal(hits_host.view(torch.int32), hits_want):
            raise RuntimeError("host-buffer and device-buffer hits differ")
        hits_host.zero_()
        return N_RAYS / statistics.mean(t) / 1e6

    e2e_staged = e2e_pass(False)
    e2e_mrays = e2e_pass(True)
    os.environ.pop("PBRT_HOST_MAPPED", None)

    # render of the same scene: 1024x1024, 16 spp, direct lighting
    scene = GpuScene(prims, lights)
    renderer = GpuSamplerRenderer(smp, cam)
    img = torch.empty((1024, 1024, 3), dtype=torch.float32, device=dev)
    renderer.render(scene, out=img, stream=stream)
    rt = []
    for _ in range(3):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        renderer.render(scene, out=img, stream=stream)
        rt.append(time.perf_counter() - t0)
    instanced = bench_instanced(torch, dev, stream)
    c1 = bench_rmse(torch, dev, stream)
    batched = bench_batched(torch, dev, stream) if not args.skip_multi else None
    served = bench_served(torch, dev, stream) if not args.skip_multi else None
    clk.__exit__(None, None, None)

    mean_ms = statistics.mean(ms_closest)
    t_local = torch.tensor([mean_ms], device=dev)
    if ws > 1:
        torch.distributed.all_reduce(t_local, op=torch.distributed.ReduceOp.MAX)
    ms_step = float(t_local.item())
    value = ws * N_RAYS / (ms_step / 1e3) / 1e6

    out = None
    if rank == 0:
        peak, peak_kind = measured_peak()
        nthreads = os.cpu_count() or 1
        cpu_rps, cpu_dt, cpu_passes, (bpr, nodes_pr, tris_pr) = cpu_baseline_leg(prims, rays, nthreads)
        alg_bytes = bpr * N_RAYS
        achieved = alg_bytes / (mean_ms / 1e3) / 1e9
        tr = committed_traffic()
        out = {
            "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "rays_per_step": N_RAYS, "bvh": "reference SAH, 1-prim leaves",
                       "l2": "flushed between steps (256 MiB write); inputs also exceed L2",
                       "parallelism": f"replicas x{ws}", "trace_config": abi.get_trace_config()},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": (tr or {}).get("dram_bytes_per_launch"),
                         "algorithmic_bytes_per_ray": bpr, "nodes_tested_per_ray": nodes_pr,
                         "tris_tested_per_ray": tris_pr},
            "cpu_baseline": {"value": cpu_rps / 1e6, "unit": "Mrays/s", "cores": nthreads, "kind": "port",
                             "sample": f"{cpu_passes} passes over the 2^22 rays, {cpu_dt:.1f} s"},
            "e2e": {"value": e2e_mrays, "unit": "Mrays/s", "h2d_bytes_per_step": N_RAYS * 32,
                    "d2h_bytes_per_step": N_RAYS * 16, "host_buffers": "pinned, read and written in place",
                    "staged": {"value": e2e_staged, "unit": "Mrays/s",
                               "how": "PBRT_HOST_MAPPED=0: H2D copy, traversal, D2H copy in 4 overlapped pieces"}},
            # per timed step: the traversal kernel and the replay check (D24)
            "gpu_launches": 2 * args.steps,
            "clocks": clk.summary(),
            "any_hit": {"value": N_RAYS / (statistics.mean(ms_any) / 1e3) / 1e6, "unit": "Mrays/s"},
            "render_1024x1024_16spp": {"ms_mean": 1e3 * statistics.mean(rt), "ms_min": 1e3 * min(rt),
                                       "camera_rays": 1024 * 1024 * 16},
            "render_c1_512x512_4spp": c1,
            "bvh_build": {"host_s": build_s, "device_s": dbuild_s, "identical": same_tree,
                          "what": "pbrtgpu_bvh_create(_ex) of the 1M-triangle heightfield, host vs device tree build"},
            "instancing": instanced,
            "batched_multi_scene": batched,
            "served": served,
        }
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--skip-multi", action="store_true", help="skip the batched and served sections")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
