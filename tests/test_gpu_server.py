"""The serving loop: continuous batching must give every request the result
it gets alone (bit for bit), whatever else shares its batch or the device,
for requests submitted from several threads while others run."""
import random
import threading

import numpy as np
import pytest

from pbrt_rust_gb300 import abi, generators as G
from pbrt_rust_gb300.gpu import GpuBVHAccel, GpuSamplerRenderer, GpuScene
from pbrt_rust_gb300.server import GpuServer

pytestmark = pytest.mark.gpu

SMALL = dict(tri_range=(500, 8000), res_choices=(16, 32, 48), spp_choices=(1, 4), max_spheres=5)


def bits(a):
    a = np.ascontiguousarray(a.cpu().numpy() if hasattr(a, "cpu") else a)
    return a.view(np.uint8).reshape(-1)


@pytest.fixture(scope="module")
def pool():
    """Five resident scenes, renders of each at two camera positions, and
    ray batches against their BVHs - each with its result alone."""
    torch = pytest.importorskip("torch")
    reqs = []
    scenes = []
    for i in range(5):
        prims, lights, cam, smp = G.multi_scene(i, seed=500 + i, **SMALL)
        sc = GpuScene(prims, lights)
        scenes.append(sc)
        reqs.append(("render", sc, GpuSamplerRenderer(smp, cam)))
        cam2 = G.orbit_camera(cam, radius=3.0 + i, azimuth=0.7 * i)
        reqs.append(("render", sc, GpuSamplerRenderer(smp, cam2)))
        lo, hi = sc.aggregate().world_bound()
        rays = G.incoherent_rays(G.PCG32(900 + i), 3000 + 1000 * i, lo, hi)
        if i % 2:
            rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
        reqs.append(("query", sc.aggregate(), rays, i % 3 == 0))
    alone = []
    for r in reqs:
        if r[0] == "render":
            alone.append(r[2].render(r[1]))
        else:
            alone.append(r[1].intersect_p(r[2]) if r[3] else r[1].intersect(r[2]))
    torch.cuda.synchronize()
    return reqs, alone, scenes


def submit(server, r):
    if r[0] == "render":
        return server.submit_render(r[1], r[2])
    return server.submit_query(r[1], r[2], any_hit=r[3])


@pytest.mark.parametrize("slots,max_samples", [(2, 1 << 16), (3, 6000), (1, 1 << 16)])
def test_results_equal_alone_in_any_mix(pool, slots, max_samples):
    torch = pytest.importorskip("torch")
    reqs, alone, _ = pool
    server = GpuServer(slots=slots, max_jobs=8, max_samples=max_samples, max_film_pixels=1 << 14,
                       max_query_rays=1 << 15, max_tasks=512)
    order = [k for k in range(len(reqs)) for _ in range(3)]
    random.Random(slots).shuffle(order)
    tickets = [None] * len(order)

    def feed(part):
        rng = random.Random(len(part))
        for pos in part:
            tickets[pos] = submit(server, reqs[order[pos]])
            if rng.random() < 0.3:
                threading.Event().wait(0.0005)

    threads = [threading.Thread(target=feed, args=(list(range(t, len(order), 2)),)) for t in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    outs = [server.wait(t) for t in tickets]
    torch.cuda.synchronize()
    for pos, out in enumerate(outs):
        assert np.array_equal(bits(out), bits(alone[order[pos]])), (pos, order[pos])
    st = server.stats()
    assert st["completed"] == st["submitted"] == len(order) and st["failed"] == 0
    assert st["p99_ms"] >= st["p50_ms"] > 0 and st["batches"] >= 1
    server.close()


def test_oversized_request_is_refused(pool):
    reqs, _, _ = pool
    server = GpuServer(slots=1, max_jobs=4, max_samples=100, max_film_pixels=1 << 12)
    with pytest.raises(abi.PbrtError) as e:
        server.submit_render(reqs[0][1], reqs[0][2])
    assert e.value.status == 7
    server.close()


def test_flood_is_batched(pool):
    """Submitted all at once, requests share batches."""
    reqs, alone, _ = pool
    server = GpuServer(slots=2, max_jobs=32, max_samples=1 << 17, max_film_pixels=1 << 15,
                       max_query_rays=1 << 16, max_tasks=1024)
    tickets = [submit(server, reqs[k % len(reqs)]) for k in range(60)]
    server.drain()
    for k, t in enumerate(tickets):
        assert np.array_equal(bits(server.wait(t)), bits(alone[k % len(reqs)]))
    st = server.stats()
    assert st["mean_batch_requests"] > 1.5, st
    server.close()


def test_pool_budget_admits_scenes_and_refuses_others(pool):
    """With a device-memory pool the slots and the resident scenes share the
    budget: a scene that does not fit is refused, requests may only name
    resident scenes or their BVHs, and served results stay the ones alone."""
    from pbrt_rust_gb300.batch import batch_bytes
    reqs, alone, scenes = pool
    lim = dict(max_jobs=64, max_samples=1 << 16, max_film_pixels=1 << 14, max_query_rays=1 << 15, max_tasks=1 << 10)
    slot = batch_bytes(**lim)[0]
    sizes = [sc.device_bytes() for sc in scenes]
    assert all(s > 0 for s in sizes)
    out = min(range(len(scenes)), key=lambda k: sizes[k])  # the scene left out: the smallest
    kept = [k for k in range(len(scenes)) if k != out]
    budget = 2 * slot + sum(sizes[k] for k in kept)  # full once the others are resident
    srv = GpuServer(slots=2, pool_bytes=budget, **lim)
    try:
        for k in kept:
            srv.admit(scenes[k])
        with pytest.raises(abi.PbrtError) as e:
            srv.admit(scenes[out])
        assert e.value.status == abi.PBRT_ERR_BUDGET
        st = srv.stats()
        assert st["pool_bytes"] == budget and st["slot_bytes"] == 2 * slot
        assert st["resident_bytes"] == sum(sizes[k] for k in kept) and st["resident_count"] == len(kept)
        tickets = []
        for r, want in zip(reqs, alone):
            sc_index = next(k for k, sc in enumerate(scenes) if (r[1] is sc or getattr(r[1], "_owner", None) is sc))
            if sc_index == out:
                with pytest.raises(abi.PbrtError) as e:
                    submit(srv, r)
                assert e.value.status == abi.PBRT_ERR_BUDGET
            else:
                tickets.append((submit(srv, r), want))
        for t, want in tickets:
            assert np.array_equal(bits(srv.wait(t)), bits(want))
        assert srv.stats()["refused"] == 3  # the left-out scene's two renders and query
        srv.release(scenes[kept[0]])
        srv.admit(scenes[out])  # it fits in the room of any larger scene
        assert srv.stats()["resident_bytes"] == sum(sizes[k] for k in kept[1:]) + sizes[out]
    finally:
        srv.close()
