"""Benchmark: closest-hit rays/s on the 1M-triangle heightfield.

Workload (the configuration the headline metric is quoted on): a
708x708-vertex heightfield (999,698 triangles) plus its 2-triangle area
light, SAH BVH built with the reference's algorithm, and 2^22 incoherent
rays (origins uniform in the mesh bounds inflated by 1, directions uniform
on the sphere).  One step = one closest-hit pass over all 2^22 rays.

  value       device-resident rays/hits, kernel time from CUDA events on
              the launching stream; L2 flushed (256 MiB write) between steps
  e2e         the same pass through the C ABI with pinned HOST buffers and
              the synchronisation inside the timed step, in the library's
              default form (streamed: one traversal launch whose warps wait
              for the ray pieces copied in behind it, the hits written to
              the host by the walk chunk by chunk); `e2e.forms` also times
              the copy pipeline (PBRT_STREAM_IN=0: copies in, traversal and
              copies out in four overlapped pieces) and PBRT_HOST_MAPPED=1,
              where the traversal reads the rays from and writes the hits to
              the mapped host memory (Grace memory over NVLink-C2C), in
              alternating rounds; `e2e.any_hit_forms` the same for any hit
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
    """dram__bytes_read.sum + dram__bytes_write.sum, warp instructions and
    lanes active per instruction of one closest-hit launch on this workload,
    from the committed ncu summary (None without one)."""
    p = ROOT / "profiles" / "k_trace4_persistent_heightfield_4M_rays.md"
    if p.exists():
        text = p.read_text()
        m = re.search(r"^dram_bytes_per_launch = (\d+)$", text, re.M)
        if m:
            out = {"dram_bytes_per_launch": int(m.group(1)), "source": str(p.relative_to(ROOT))}
            w = re.search(r"^warp_instructions_per_launch = (\d+)$", text, re.M)
            a = re.search(r"^lanes_active_per_instruction = ([0-9.]+)$", text, re.M)
            if w and a:
                out["warp_instructions_per_launch"] = int(w.group(1))
                out["lanes_active_per_instruction"] = float(a.group(1))
            return out
    return None


def issue_view(torch, tr, mean_ms, clocks):
    """What bounds the headline kernel: its warp instructions per launch
    (committed ncu summary) over this run's launch time, against the issue
    peak of the device at the median SM clock of this run (one instruction
    per scheduler per cycle, 4 schedulers per SM), and the lanes active per
    instruction."""
    if not tr or "warp_instructions_per_launch" not in tr or not clocks.get("sm_mhz"):
        return None
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    rate = tr["warp_instructions_per_launch"] / (mean_ms / 1e3)
    peak = sms * 4 * clocks["sm_mhz"] * 1e6
    lanes = tr["lanes_active_per_instruction"]
    return {"warp_instructions_per_s": rate, "peak": peak, "frac": rate / peak, "lanes_active": lanes,
            "thread_frac": rate / peak * lanes / 32.0, "source": tr["source"]}


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


SWEEP_RATES = (50.0, 200.0, 500.0, 1000.0, 2000.0)
POOL_BYTES = 120 * 10**9  # the serving workload's device-memory budget


def bench_served(torch, dev, stream, n_scenes: int = 32, n_requests: int = 2000, rates=SWEEP_RATES, slots: int = 2):
    """Requests/s and latency of the serving loop against the plain path
    (one request at a time through pbrtgpu_render / pbrtgpu_intersect) on
    the same request stream; all outputs device-resident.  The server holds
    the resident scenes and its slots in a 120 GB device-memory pool; the
    flood submits every request at once, the sweep submits them as Poisson
    arrivals at each rate."""
    from pbrt_rust_gb300 import generators as G
    from pbrt_rust_gb300.profile import run_plain, run_served, serving_pool, serving_requests
    from pbrt_rust_gb300.server import GpuServer

    from pbrt_rust_gb300 import abi
    pool = serving_pool(n_scenes)
    reqs = serving_requests(pool, n_requests, dev)
    # the plain path with each render kernel (identical outputs): the
    # library's default and the 4-wide walk, which these scenes favour
    before = abi.get_trace_config()
    plain_s, plain_lat = {}, {}
    for rk in ("plain", "w4"):
        abi.set_trace_config(render_kernel=rk)
        run_plain(reqs[:20], stream)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        plain_lat[rk] = run_plain(reqs, stream)
        plain_s[rk] = time.perf_counter() - t0
    abi.set_trace_config(**before)
    default_rk = before["render_kernel"] if before["render_kernel"] in plain_s else "plain"

    def pct(lat, q):  # milliseconds
        return float(np.percentile(np.asarray(lat) * 1e3, q))
    ref = [r[3].clone() for r in reqs]
    srv = GpuServer(slots=slots, pool_bytes=POOL_BYTES, max_jobs=256, max_samples=1 << 24, max_film_pixels=1 << 22,
                    max_query_rays=1 << 20, max_tasks=1 << 14)
    for sc, _, _ in pool:
        srv.admit(sc)
    outs = [torch.empty_like(r[3]) for r in reqs]
    run_served(srv, reqs, outs)
    flood = run_served(srv, reqs, outs)
    torch.cuda.synchronize(dev)
    exact = all(torch.equal(a.view(torch.int32), b.view(torch.int32)) for a, b in zip(outs, ref))
    if not exact:
        raise RuntimeError("served results differ from the one-request results")
    sweep = []
    for k, rate in enumerate(rates):
        arrivals = G.poisson_arrivals(len(reqs), rate, seed=9 + k)
        st = run_served(srv, reqs, outs, arrivals)
        # the plain path under the same arrivals: one request at a time, a
        # request waiting while the one before it runs
        lat = run_plain(reqs, stream, arrivals)
        sweep.append({"rate": rate, "requests": st["completed"], "requests_per_s": st["requests_per_s"],
                      "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
                      "max_ms": st["max_ms"], "mean_batch": st["mean_batch_requests"], "deferred": st["deferred"],
                      "refused": st["refused"], "plain_p50_ms": pct(lat, 50), "plain_p99_ms": pct(lat, 99),
                      "plain_mean_ms": float(np.mean(lat) * 1e3)})
    final = srv.stats()
    srv.close()
    n_render = sum(1 for r in reqs if r[0] == "render")
    return {"scenes": n_scenes, "requests": len(reqs), "renders": n_render, "queries": len(reqs) - n_render,
            "slots": slots, "plain_requests_per_s": len(reqs) / plain_s[default_rk],
            "plain_requests_per_s_by_render_kernel": {k: len(reqs) / v for k, v in plain_s.items()},
            "served_requests_per_s": flood["requests_per_s"],
            "speedup": flood["requests_per_s"] * plain_s[default_rk] / len(reqs),
            "speedup_vs_fastest_plain": flood["requests_per_s"] * min(plain_s.values()) / len(reqs),
            "flood_p50_ms": flood["p50_ms"], "flood_p99_ms": flood["p99_ms"],
            "plain_latency_ms": {"p50": pct(plain_lat[default_rk], 50), "p99": pct(plain_lat[default_rk], 99),
                                 "mean": float(np.mean(plain_lat[default_rk]) * 1e3),
                                 "how": "each request alone through its one-request call, back to back"},
            "flood_mean_batch": flood["mean_batch_requests"], "flood_deferred": flood["deferred"],
            "pool": {"budget_bytes": POOL_BYTES, "slot_bytes": final["slot_bytes"],
                     "resident_bytes": final["resident_bytes"], "resident_scenes": final["resident_count"],
                     "admitted": "all scenes; requests name resident scenes only",
                     "deferred_means": "a request found the free slot full and waited for the next one"},
            "sweep": sweep, "bit_exact": exact}


def timed_events(torch, stream, flush, fn, steps: int, warmup: int):
    """CUDA-event times (ms) of `steps` calls of fn on `stream` after
    `warmup` untimed ones, the L2 flushed (256 MiB write) before each."""
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            flush.zero_()
            fn()
    torch.cuda.synchronize()
    evs = []
    with torch.cuda.stream(stream):
        for _ in range(steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            evs.append((a, b))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in evs]


def l2_copy_gbs(torch, dev, stream, mib: int = 16, reps: int = 200) -> float:
    """Copy bandwidth within L2 measured here: a 16 MiB buffer copied to
    another 200 times back to back (both stay L2-resident), read + write
    bytes over the CUDA-event time.  The L2 peak the L2-resident workloads
    are compared with."""
    a = torch.empty(mib << 20, dtype=torch.uint8, device=dev)
    b = torch.empty_like(a)
    with torch.cuda.stream(stream):
        for _ in range(20):
            b.copy_(a)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            b.copy_(a)
        e1.record(stream)
    torch.cuda.synchronize(dev)
    return 2.0 * a.numel() * reps / (e0.elapsed_time(e1) / 1e3) / 1e9


def bench_c0(torch, dev, stream, flush, steps: int, warmup: int):
    """The plain ray-BVH query workload: 4096 random triangles (SAH BVH,
    ~0.5 MB, L2-resident) and 2^20 rays toward the centre, closest and any
    hit, device-resident buffers, L2 flushed before each step."""
    from pbrt_rust_gb300 import abi, generators as G
    from pbrt_rust_gb300.gpu import GpuBVHAccel
    lib = abi.load()
    prims, rays = G.ray_soup(4096, 1 << 20)
    n = len(rays)
    bvh = GpuBVHAccel(prims, 4, "sah")
    sh = C.c_void_p(stream.cuda_stream)
    rd = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
    hd = torch.empty((n, 4), dtype=torch.float32, device=dev)
    od = torch.empty((n,), dtype=torch.uint8, device=dev)
    rp, hp, op = C.c_void_p(rd.data_ptr()), C.c_void_p(hd.data_ptr()), C.c_void_p(od.data_ptr())
    ms_c = timed_events(torch, stream, flush, lambda: abi.check(lib.pbrtgpu_intersect(bvh._h, rp, n, hp, sh), lib),
                        steps, warmup)
    ms_a = timed_events(torch, stream, flush, lambda: abi.check(lib.pbrtgpu_intersect_p(bvh._h, rp, n, op, sh), lib),
                        steps, warmup)
    out = {"workload": "4096 random triangles (SAH, 1-prim leaves) + 2^20 rays toward the centre",
           "rays": n, "closest": {"ms": statistics.mean(ms_c), "mrays_s": n / statistics.mean(ms_c) / 1e3},
           "any": {"ms": statistics.mean(ms_a), "mrays_s": n / statistics.mean(ms_a) / 1e3},
           "bvh_device_bytes": bvh.device_bytes(), "l2": "flushed before each step (256 MiB write)"}
    return out, (prims, rays)


def bench_render(torch, dev, stream, flush, prims, lights, cam, smp, frames: int = 5):
    """Frames of the direct-lighting wavefront through pbrtgpu_render
    (device output): CUDA-event time on the stream and wall time of the
    call (which returns once the frame is done), L2 flushed before each."""
    from pbrt_rust_gb300.gpu import GpuSamplerRenderer, GpuScene
    scene = GpuScene(prims, lights)
    r = GpuSamplerRenderer(smp, cam)
    x0, x1, y0, y1 = cam.film.pixel_extent()
    img = torch.empty((y1 - y0, x1 - x0, 3), dtype=torch.float32, device=dev)
    r.render(scene, out=img, stream=stream)
    ev, wall = [], []
    for _ in range(frames):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize(dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        a.record(stream)
        r.render(scene, out=img, stream=stream)
        b.record(stream)
        wall.append(time.perf_counter() - t0)
        torch.cuda.synchronize(dev)
        ev.append(a.elapsed_time(b))
    spp = smp.x_samples * smp.y_samples
    samples = (x1 - x0) * (y1 - y0) * spp
    ms = statistics.mean(ev)
    return {"ms_mean": ms, "ms_min": min(ev), "wall_ms_mean": 1e3 * statistics.mean(wall),
            "images_per_s": 1e3 / ms, "samples_per_s": samples / (ms / 1e3), "samples": samples, "spp": spp,
            "camera_rays": samples, "l2": "flushed before each frame"}, img


def render_bytes(stats, samples: int) -> float:
    """Algorithmic bytes of a frame from the oracle's counts of the same
    frame (camera rays, shadow rays, then nodes / triangles / analytic
    shapes tested by camera rays and by shadow rays): per camera ray 32 B
    ray + 16 B hit + 32 B per node + 48 B per triangle + 16 B per analytic
    shape tested, 16 B of material and 16 B of film per sample; per shadow
    ray 32 B ray + 1 B answer + its nodes, triangles and shapes."""
    cam, shadow, cn, ct, cs, sn, stt, ss = (float(x) for x in stats[:8])
    return (cam * (32 + 16) + 32 * cn + 48 * ct + 16 * cs + samples * (16 + 16)
            + shadow * (32 + 1) + 32 * sn + 48 * stt + 16 * ss)


def cpu_render_leg(prims, lights, cam, smp, num_tasks: int, nthreads: int, single_tasks, min_seconds: float = 3.0):
    """The oracle renderer (SamplerRenderer::render restated, the reference's
    task split and per-task sub-films, one std::thread worker per host
    thread taking whole tasks) on the same frame: whole frames with every
    host thread until min_seconds have passed, and the tasks
    `single_tasks` on one thread.  The scene is built once, untimed.
    Returns (frames/s, samples/s all threads, samples/s one thread,
    seconds, frames, single-thread samples and seconds, the oracle's work
    counts of one frame)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    from pbrt_rust_gb300.scene import SceneDescription
    sc = O.OracleScene(SceneDescription(prims, lights))
    x0, x1, y0, y1 = cam.film.pixel_extent()
    spp = smp.x_samples * smp.y_samples
    frame_samples = (x1 - x0) * (y1 - y0) * spp
    frames, t0 = 0, time.perf_counter()
    stats = None
    while True:
        _, st = sc.render(cam, smp, num_tasks, nthreads=nthreads)
        stats = st if stats is None else stats
        frames += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            break
    one_samples, t1 = 0, time.perf_counter()
    for t in single_tasks:
        _, st = sc.render(cam, smp, num_tasks, nthreads=1, task_lo=t, task_hi=t + 1)
        one_samples += int(st[0])
    one_dt = time.perf_counter() - t1
    return (frames / dt, frames * frame_samples / dt, one_samples / one_dt, dt, frames, one_samples, one_dt, stats)


def render_report(gpu: dict, cpu, num_tasks: int, nthreads: int, single_tasks, peak: float, l2_gbs: float) -> dict:
    fps, sps, sps1, dt, frames, one_samples, one_dt, stats = cpu
    alg = render_bytes(stats, gpu["samples"])
    achieved = alg / (gpu["ms_mean"] / 1e3) / 1e9
    out = dict(gpu)
    out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                       "l2_peak": l2_gbs, "l2_frac": achieved / l2_gbs, "algorithmic_bytes_per_frame": alg,
                       "algorithmic_bytes_per_sample": alg / gpu["samples"],
                       "counts": {"camera_rays": int(stats[0]), "shadow_rays": int(stats[1]),
                                  "camera_nodes": int(stats[2]), "camera_tris": int(stats[3]),
                                  "camera_shapes": int(stats[4]), "shadow_nodes": int(stats[5]),
                                  "shadow_tris": int(stats[6]), "shadow_shapes": int(stats[7])},
                       "how": "oracle counts of this frame in the reference traversal order; 32 B/node, 48 B/"
                              "triangle, 16 B/shape, rays, hits, 16 B material + 16 B film per sample"}
    out["cpu_baseline"] = {"images_per_s": fps, "samples_per_s": sps, "unit": "images/s", "value": fps,
                           "cores": nthreads, "hardware_concurrency": os.cpu_count(), "num_tasks": num_tasks,
                           "kind": "port", "sample": f"{frames} whole frames in {dt:.1f} s, all host threads "
                           f"(the reference's {num_tasks}-task split bounds the parallelism)",
                           "single_thread": {"samples_per_s": sps1, "images_per_s": sps1 / gpu["samples"],
                                             "cores": 1, "sample": f"tasks {list(single_tasks)} of {num_tasks}: "
                                             f"{one_samples} samples in {one_dt:.1f} s"}}
    return out


# single-thread CPU samples: every third task of the frame's task split
C2_SINGLE_TASKS = (2, 5, 8, 11)   # of the 12 tasks of 1024 x 1024
C1_SINGLE_TASKS = (1, 4, 7)       # of the 10 tasks of 512 x 512


def c0_report(c0: dict, data, nthreads: int, peak: float, l2_gbs: float, min_seconds: float = 3.0) -> dict:
    """Rooflines and CPU baseline of the plain query workload: algorithmic
    bytes per ray counted by the oracle's reference-order traversal of all
    2^20 rays (32 B per node, 48 B per triangle, 32 B ray, 16 B hit or 1 B
    answer; any hit counted to its first accepted primitive, as the device
    walks it) over the CUDA-event time, against the measured HBM copy
    bandwidth and the L2 copy bandwidth measured in this run (the BVH is
    L2-resident); the oracle's whole passes over the rays on every host
    thread for the CPU figure."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    prims, rays = data
    ob = O.OracleBVH(prims, 4, "sah")
    rays = np.ascontiguousarray(rays)
    n = len(rays)
    _, cnt = ob.intersect(rays, counters=True, nthreads=nthreads)
    _, cnt_any = ob.first_hit_counts(rays, nthreads=nthreads)
    out = dict(c0)
    for key, k, res_bytes in (("closest", cnt, 16.0), ("any", cnt_any, 1.0)):
        bpr = (32.0 * k[0] + 48.0 * k[1] + 16.0 * k[2]) / n + 32.0 + res_bytes
        ach = bpr * n / (c0[key]["ms"] / 1e3) / 1e9
        out[key]["roofline"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                                "l2_peak": l2_gbs, "l2_frac": ach / l2_gbs, "algorithmic_bytes_per_ray": bpr,
                                "nodes_tested_per_ray": float(k[0]) / n, "tris_tested_per_ray": float(k[1]) / n}
    passes, t0 = 0, time.perf_counter()
    while True:
        ob.intersect(rays, nthreads=nthreads)
        passes += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            break
    out["cpu_baseline"] = {"value": passes * n / dt / 1e6, "unit": "Mrays/s", "cores": nthreads, "kind": "port",
                           "sample": f"{passes} closest-hit passes over the 2^20 rays, {dt:.1f} s"}
    return out


def bench_rmse(torch, dev, stream, flush):
    """The plain render config (512x512, 2x2 strata, ground, 64 spheres,
    point + area light): frame time (bench_render) and RMSE (linear RGB)
    against the same scene at 8x8 strata (64 spp, the most a pixel takes;
    same task split, so the same task seams), whose own noise adds about 3 %
    to the figure.  The batched and served forms produce bit-identical
    images, hence the same RMSE."""
    from pbrt_rust_gb300 import generators as G
    from pbrt_rust_gb300.gpu import GpuSamplerRenderer, GpuScene
    prims, lights, cam, smp = G.c1_scene(res=512)
    out, img = bench_render(torch, dev, stream, flush, prims, lights, cam, smp, frames=10)
    _, _, _, smp64 = G.c1_scene(res=512, spp_side=8)
    ref = torch.empty_like(img)
    GpuSamplerRenderer(smp64, cam).render(GpuScene(prims, lights), out=ref, stream=stream)
    torch.cuda.synchronize(dev)
    out["rmse_vs_64spp"] = float(torch.sqrt(torch.mean((img - ref) ** 2)).item())
    out["reference_mean"] = float(ref.mean().item())
    return out, (prims, lights, cam, smp)


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
    # e2e: pinned host buffers through the C ABI, staged through device
    # copies (default, PBRT_HOST_MAPPED=0) or read and written in place (=1)
    rays_host = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
    hits_host = torch.empty((N_RAYS, 4), dtype=torch.float32).pin_memory()
    rh, hh = C.c_void_p(rays_host.data_ptr()), C.c_void_p(hits_host.data_ptr())
    torch.cuda.synchronize(dev)
    hits_want = hits_dev.cpu().view(torch.int32)

    occ_host = torch.empty((N_RAYS,), dtype=torch.uint8).pin_memory()
    oh = C.c_void_p(occ_host.data_ptr())
    occ_want = occ_dev.cpu()
    form_env = {"default": {}, "pipelined": {"PBRT_STREAM_IN": "0"}, "in_place": {"PBRT_HOST_MAPPED": "1"}}

    def e2e_pass(form, any_hit=False) -> float:
        for k in ("PBRT_STREAM_IN", "PBRT_HOST_MAPPED"):
            os.environ.pop(k, None)
        os.environ.update(form_env[form])

        def call():
            if any_hit:
                abi.check(lib.pbrtgpu_intersect_p(bvh._h, rh, N_RAYS, oh, sh), lib)
            else:
                abi.check(lib.pbrtgpu_intersect(bvh._h, rh, N_RAYS, hh, sh), lib)
        for _ in range(args.warmup):
            call()
        t = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            call()
            t.append(time.perf_counter() - t0)
        # the host copy of the result must equal the device-resident one
        if not (torch.equal(occ_host, occ_want) if any_hit else torch.equal(hits_host.view(torch.int32), hits_want)):
            raise RuntimeError(f"host-buffer and device-buffer results differ ({form})")
        hits_host.zero_()
        occ_host.fill_(7)
        return N_RAYS / statistics.mean(t) / 1e6

    # the default and the other host-buffer forms alternate over a few rounds
    runs = {k: [] for k in form_env}
    any_runs = {k: [] for k in form_env}
    for _ in range(4):
        for k in form_env:
            runs[k].append(e2e_pass(k))
            any_runs[k].append(e2e_pass(k, any_hit=True))
    e2e_mrays = statistics.median(runs["default"])
    for k in ("PBRT_STREAM_IN", "PBRT_HOST_MAPPED"):
        os.environ.pop(k, None)

    # render of the same scene: 1024x1024, 16 spp, direct lighting
    c2, _ = bench_render(torch, dev, stream, flush, prims, lights, cam, smp, frames=5)
    c1, c1_scene = bench_rmse(torch, dev, stream, flush)
    c0, c0_data = bench_c0(torch, dev, stream, flush, args.steps, args.warmup)
    l2_gbs = l2_copy_gbs(torch, dev, stream)
    instanced = bench_instanced(torch, dev, stream)
    batched = bench_batched(torch, dev, stream) if not args.skip_multi else None
    served = bench_served(torch, dev, stream, n_requests=args.requests) if not args.skip_multi else None
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
        from pbrt_rust_gb300.scene import default_num_tasks
        nt_c2 = default_num_tasks(1024, 1024)
        cpu_c2 = cpu_render_leg(prims, lights, cam, smp, nt_c2, nthreads, C2_SINGLE_TASKS)
        nt_c1 = default_num_tasks(512, 512)
        cpu_c1 = cpu_render_leg(*c1_scene, nt_c1, nthreads, C1_SINGLE_TASKS)
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
                         "tris_tested_per_ray": tris_pr,
                         "issue": issue_view(torch, tr, mean_ms, clk.summary())},
            "cpu_baseline": {"value": cpu_rps / 1e6, "unit": "Mrays/s", "cores": nthreads, "kind": "port",
                             "sample": f"{cpu_passes} passes over the 2^22 rays, {cpu_dt:.1f} s"},
            "e2e": {"value": e2e_mrays, "unit": "Mrays/s", "h2d_bytes_per_step": N_RAYS * 32,
                    "d2h_bytes_per_step": N_RAYS * 16,
                    "how": "median of 4 rounds of the library's default form, pinned host buffers",
                    "forms": {k: {"median": statistics.median(v), "min": min(v), "max": max(v), "runs": v}
                              for k, v in runs.items()},
                    "any_hit_forms": {k: {"median": statistics.median(v), "min": min(v), "max": max(v)}
                                      for k, v in any_runs.items()},
                    "form_meaning": {"default": "streamed: one traversal launch; the rays follow in pieces on a "
                                                "copy stream and warps wait for the piece they take; closest hits "
                                                "are staged on the device and written to the host by the walk, "
                                                "chunk by chunk in coalesced rows",
                                     "in_place": "PBRT_HOST_MAPPED=1: the traversal reads the rays from and "
                                                 "writes the hits to the mapped host memory",
                                     "pipelined": "PBRT_STREAM_IN=0: H2D copy, traversal, D2H copy in 4 "
                                                  "overlapped pieces"}},
            # per timed step: the traversal kernel and the replay check (D24)
            "gpu_launches": 2 * args.steps,
            "clocks": clk.summary(),
            "any_hit": {"value": N_RAYS / (statistics.mean(ms_any) / 1e3) / 1e6, "unit": "Mrays/s"},
            "render_1024x1024_16spp": render_report(c2, cpu_c2, nt_c2, nthreads, C2_SINGLE_TASKS, peak, l2_gbs),
            "render_c1_512x512_4spp": render_report(c1, cpu_c1, nt_c1, nthreads, C1_SINGLE_TASKS, peak, l2_gbs),
            "c0_soup_4096_tris_2e20_rays": c0_report(c0, c0_data, nthreads, peak, l2_gbs),
            "l2_copy_gbs": {"value": l2_gbs, "how": "16 MiB buffer copied 200 times within L2, read + write bytes, "
                                                    "CUDA events (measured in this run)"},
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
    ap.add_argument("--requests", type=int, default=2000, help="requests of the served section (flood and each rate)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: relaunch under torch.distributed.run (what a
        # torchrun launch does), each rank tracing its own rays against a
        # replicated BVH; rank 0 prints the line
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr", "127.0.0.1", "--master-port", str(port), str(Path(__file__).resolve()),
               *sys.argv[1:]]
        return subprocess.call(cmd)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
