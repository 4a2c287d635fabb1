"""GPU parity of TransformedPrimitive instances (nested traversal of the
definitions' BVHs) against the CPU oracle's two-level restatement
(src/primitive/transformed.rs:35-59).

Triangle and full-quadric definitions give bit-identical hits; renders match
within the render tests' 1e-4 (sphere normals go through acosf/sinf)."""
import numpy as np
import pytest

from pbrt_rust_gb300 import abi, generators as G
from pbrt_rust_gb300.batch import GpuBatch
from pbrt_rust_gb300.gpu import GpuBVHAccel, GpuSamplerRenderer, GpuScene
from pbrt_rust_gb300.scene import SceneDescription, default_num_tasks

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("device_build", [False, True])
def test_instance_queries_are_bit_exact(oracle, device_build):
    prims, _, _, _, _ = G.instanced_forest(n_instances=40, tris_per_tree=800, seed=11)
    rays = G.rays_toward_center(G.PCG32(5), 1 << 16, radius=14.0, target=4.0)
    g = GpuBVHAccel(prims, 4, "sah", build_on_device=device_build)
    o = oracle.OracleBVH(prims, 4, "sah")
    want = o.intersect(rays)
    assert (want["prim"] >= 0).sum() > 10000
    assert np.array_equal(g.intersect(rays).view(np.uint32), want.view(np.uint32))
    assert np.array_equal(g.intersect_p(rays), o.intersect_p(rays))


def test_instance_queries_from_pinned_host_memory(oracle):
    """Pinned host rays on a tree with instances take the streamed form
    (the instanced walk waiting for ray pieces, closest hits written out
    chunk by chunk): the answers equal the oracle's bit for bit."""
    import torch
    prims, _, _, _, _ = G.instanced_forest(n_instances=24, tris_per_tree=500, seed=12)
    n = (1 << 17) + 999
    rays = G.rays_toward_center(G.PCG32(6), n, radius=14.0, target=4.0)
    g = GpuBVHAccel(prims, 4, "sah")
    o = oracle.OracleBVH(prims, 4, "sah")
    want = o.intersect(rays)
    assert (want["prim"] >= 0).sum() > 10000
    pinned = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
    out = torch.full((n, 4), 7.0, dtype=torch.float32).pin_memory()
    g.intersect(pinned, out=out)
    assert np.array_equal(out.numpy().view(np.uint32).reshape(-1), want.view(np.uint32).reshape(-1))
    occ = torch.full((n,), 9, dtype=torch.uint8).pin_memory()
    g.intersect_p(pinned, out=occ)
    assert np.array_equal(occ.numpy(), o.intersect_p(rays))


def test_instance_ids_cover_every_definition_primitive(oracle):
    """Hits land inside many instances and on primitives of both
    definitions; ids stay below the counted-out total."""
    prims, _, _, _, _ = G.instanced_forest(n_instances=16, tris_per_tree=200, seed=2)
    total = SceneDescription(prims, [], aggregate_only=True).num_ids()
    rays = G.rays_toward_center(G.PCG32(9), 1 << 15, radius=14.0, target=4.0)
    h = GpuBVHAccel(prims).intersect(rays)
    ids = h["prim"][h["prim"] >= 0]
    assert ids.max() < total and len(np.unique(ids)) > 100
    first = np.cumsum([0] + [p.shape.num_ids() for p in prims])[:-1]
    owner = np.searchsorted(first, ids, side="right") - 1
    assert sum(prims[k].shape.kind == abi.SHAPE_INSTANCE for k in set(owner.tolist())) == 16


def test_instanced_render_matches_oracle(oracle):
    prims, lights, cam, smp, _ = G.instanced_forest(n_instances=32, tris_per_tree=600, seed=4, res=96)
    nt = default_num_tasks(cam.film.x_res, cam.film.y_res)
    gpu = GpuSamplerRenderer(smp, cam, num_tasks=nt).render(GpuScene(prims, lights, 4, "sah"))
    ref = oracle.render(SceneDescription(prims, lights, 4, "sah"), cam, smp, nt)
    assert np.isfinite(gpu).all() and ref.max() > 0.1
    diff = np.abs(gpu - ref)
    assert diff.max() <= 1e-4, (diff.max(), np.unravel_index(diff.argmax(), diff.shape))


def test_instanced_render_in_a_batch_equals_the_single_render():
    """Batch kernels take the instance-aware walk for such jobs; the image
    of an instanced scene next to a plain one is the single render's."""
    prims, lights, cam, smp, _ = G.instanced_forest(n_instances=12, tris_per_tree=300, seed=6, res=64)
    p2, l2, c2, s2 = G.c1_scene(res=64, n_spheres=8)
    a, b = GpuScene(prims, lights), GpuScene(p2, l2)
    nt = default_num_tasks(64, 64)
    ra, rb = GpuSamplerRenderer(smp, cam, num_tasks=nt), GpuSamplerRenderer(s2, c2, num_tasks=nt)
    alone, alone2 = ra.render(a), rb.render(b)
    queries = G.rays_toward_center(G.PCG32(3), 4096, radius=14.0, target=4.0)
    bvh = GpuBVHAccel(prims)
    batch = GpuBatch(max_jobs=8, max_samples=1 << 16, max_query_rays=1 << 13)
    batch.add_render(a, ra)
    batch.add_render(b, rb)
    batch.add_query(bvh, queries)
    out = batch.run()
    assert np.array_equal(out[0].view(np.uint32), alone.view(np.uint32))
    assert np.array_equal(out[1].view(np.uint32), alone2.view(np.uint32))
    assert np.array_equal(out[2].view(np.uint32), bvh.intersect(queries).view(np.uint32))


def test_oren_nayar_instanced_batch_equals_the_single_render():
    """Oren-Nayar materials inside instance definitions, rendered alone and
    in a batch next to a query of the same aggregate."""
    prims, lights, cam, smp, _ = G.instanced_forest(n_instances=10, tris_per_tree=200, seed=8, res=48)
    for p in prims[1:-1]:
        for q in p.shape.definition.prims:
            q.material = type(q.material)(q.material.kd, sigma=30.0)
    sc = GpuScene(prims, lights)
    nt = default_num_tasks(48, 48)
    r = GpuSamplerRenderer(smp, cam, num_tasks=nt)
    alone = r.render(sc)
    batch = GpuBatch(max_jobs=4, max_samples=1 << 15)
    batch.add_render(sc, r)
    out = batch.run()
    assert np.array_equal(out[0].view(np.uint32), alone.view(np.uint32))
    assert alone.max() > 0.05
