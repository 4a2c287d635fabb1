"""The batched multi-scene wavefront (pbrtgpu_batch_*) against the
single-job entry points and the oracle.

Every job's output must equal what pbrtgpu_render / pbrtgpu_intersect /
pbrtgpu_intersect_p give for it alone, bit for bit, under every tuning, with
and without the CUDA graph, across launches that reuse the batch.
"""
import numpy as np
import pytest

from pbrt_rust_gb300 import abi, generators as G
from pbrt_rust_gb300.batch import GpuBatch
from pbrt_rust_gb300.gpu import GpuBVHAccel, GpuSamplerRenderer, GpuScene
from pbrt_rust_gb300.scene import SceneDescription

pytestmark = pytest.mark.gpu

SMALL = dict(tri_range=(300, 6000), res_choices=(24, 40, 56), spp_choices=(1, 4, 16), max_spheres=6)


def bits(a):
    a = np.ascontiguousarray(a.cpu().numpy() if hasattr(a, "cpu") else a)
    return a.view(np.uint8).reshape(-1)


@pytest.fixture(scope="module")
def jobs():
    """Six small scenes of the multi-scene workload with their single-job
    images, and three ray batches with their single-job hits."""
    torch = pytest.importorskip("torch")
    scenes = []
    for i in range(6):
        prims, lights, cam, smp = G.multi_scene(i, seed=1000 + i, **SMALL)
        sc = GpuScene(prims, lights)
        r = GpuSamplerRenderer(smp, cam)
        scenes.append((sc, r, r.render(sc), (prims, lights, cam, smp)))
    queries = []
    for i, (any_hit, on_dev) in enumerate([(False, False), (True, True), (False, True)]):
        prims, rays = G.ray_soup(2000 + 500 * i, 20000 + 3000 * i, seed=40 + i)
        bvh = GpuBVHAccel(prims)
        want = bvh.intersect_p(rays) if any_hit else bvh.intersect(rays)
        if on_dev:
            rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
        queries.append((bvh, rays, any_hit, want))
    return scenes, queries


def fill(batch, scenes, queries):
    for sc, r, _, _ in scenes:
        batch.add_render(sc, r)
    for bvh, rays, any_hit, _ in queries:
        batch.add_query(bvh, rays, any_hit=any_hit)


def check(outs, scenes, queries):
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    for (_, _, want, _), got in zip(scenes, outs[:len(scenes)]):
        assert np.array_equal(bits(got), bits(want))
    for (_, _, _, want), got in zip(queries, outs[len(scenes):]):
        assert np.array_equal(bits(got), bits(want))


def test_batch_equals_single_jobs(jobs):
    scenes, queries = jobs
    b = GpuBatch(max_jobs=16, max_samples=1 << 18, max_query_rays=1 << 16)
    fill(b, scenes, queries)
    st = b.stats()
    assert st["jobs"] == 9 and st["query_rays"] == sum(len(q[1]) for q in queries)
    check(b.run(), scenes, queries)
    assert max(img.max() for _, _, img, _ in scenes) > 0.05


def test_batch_render_matches_oracle(jobs, oracle):
    scenes, _ = jobs
    b = GpuBatch(max_jobs=4, max_samples=1 << 18)
    sc, r, _, (prims, lights, cam, smp) = scenes[1]
    b.add_render(sc, r)
    got = b.run()[0]
    want = oracle.render(SceneDescription(prims, lights, 4, "sah"), cam, smp, r.num_tasks)
    assert np.abs(got - want).max() <= 1e-4


@pytest.mark.parametrize("tune", [
    dict(extend_kernel="wide", shadow_kernel="wide"),
    dict(extend_kernel="wide", shadow_kernel="pair", stack=8, block=256),
    dict(extend_kernel="pair", shadow_kernel="wide", chunk=32, refill=4, refill_shadow=4),
    dict(block=256, chunk=256, refill=1, refill_shadow=16, use_graph=0),
    dict(extend_kernel="pair", shadow_kernel="pair", block=256, chunk=96, refill=32, refill_shadow=32),
])
def test_every_tuning_gives_the_same_outputs(jobs, tune):
    scenes, queries = jobs
    b = GpuBatch(max_jobs=16, max_samples=1 << 18, max_query_rays=1 << 16)
    b.set_tuning(**tune)
    for _ in range(2):  # the second launch replays the captured graph
        fill(b, scenes, queries)
        check(b.run(), scenes, queries)
    assert b.stats()["graph"] == (1 if tune.get("use_graph", 1) else 0)


def test_launches_with_different_jobs_reuse_the_batch(jobs):
    """One graph serves batches of different contents: alone, in a mix, in
    another order."""
    scenes, queries = jobs
    b = GpuBatch(max_jobs=16, max_samples=1 << 18, max_query_rays=1 << 16)
    order = [[0], [3, 1], [5, 4, 2, 0, 1], [2]]
    for sel in order:
        for i in sel:
            b.add_render(scenes[i][0], scenes[i][1])
        b.add_query(*queries[1][:2], any_hit=True)
        outs = b.run()
        for i, got in zip(sel, outs):
            assert np.array_equal(bits(got), bits(scenes[i][2]))
        assert np.array_equal(bits(outs[-1]), bits(queries[1][3]))


def test_budget_refuses_a_job_and_keeps_the_rest(jobs):
    scenes, _ = jobs
    sc, r, want, _ = scenes[0]
    n = r.pixel_extent()
    need = (n[1] - n[0]) * (n[3] - n[2]) * r.sampler.x_samples * r.sampler.y_samples
    b = GpuBatch(max_jobs=4, max_samples=need + 10, max_film_pixels=1 << 16)
    b.add_render(sc, r)
    with pytest.raises(abi.PbrtError) as e:
        b.add_render(sc, r)
    assert e.value.status == 7  # PBRT_ERR_BUDGET
    outs = b.run()
    assert len(outs) == 1 and np.array_equal(bits(outs[0]), bits(want))


def test_autotune_keeps_results(jobs):
    scenes, queries = jobs
    b = GpuBatch(max_jobs=16, max_samples=1 << 18, max_query_rays=1 << 16)
    fill(b, scenes, queries)
    tuned, ms = b.autotune(repeats=1)
    assert ms > 0 and tuned["block"] in (128, 256)
    check(b.run(), scenes, queries)


def test_thin_lens_jobs_equal_single_renders(oracle):
    """Thin-lens cameras (the sampler's general path) in one batch, with odd
    and even sample counts so that jobs start on both halves of a 16-byte
    film-position pair: each job equals its single render and the oracle."""
    from pbrt_rust_gb300.scene import Camera, StratifiedSampler
    b = GpuBatch(max_jobs=4, max_samples=1 << 18)
    want = []
    for res, side in ((33, 1), (40, 3), (24, 2)):
        prims, lights, cam0, _ = G.c1_scene(res=res, n_spheres=0)
        cam = Camera.perspective(cam0.camera_to_world, cam0.screen_window, 0.0, 1.0, 0.08, 5.5, cam0.fov, cam0.film)
        smp = StratifiedSampler.stratified(0, res, 0, res, side, side, True, 0.0, 1.0)
        sc, r = GpuScene(prims, lights, 4, "sah"), GpuSamplerRenderer(smp, cam)
        single = r.render(sc)
        ref = oracle.render(SceneDescription(prims, lights, 4, "sah"), cam, smp, r.num_tasks)
        assert np.array_equal(single.view(np.uint32), ref.view(np.uint32))
        b.add_render(sc, r)
        want.append(single)
    for got, w in zip(b.run(), want):
        assert np.array_equal(bits(got), bits(w))
