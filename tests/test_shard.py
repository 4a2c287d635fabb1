"""Sharding the path across ranks: split, run each shard, merge, compare
with the unsharded result.

World-size-2 process groups on the gloo backend, on the CPU; the per-shard
work is done by the oracle (the same algorithm the device kernels follow,
which the GPU tests check bit for bit), so this covers the split and merge
logic of pbrt_rust_gb300.shard without a GPU.
"""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

from pbrt_rust_gb300.shard import shard_range, task_range

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("n,world", [(0, 2), (1, 2), (7, 3), (1 << 20, 8), (5, 8)])
def test_shard_range_tiles(n, world):
    parts = [shard_range(n, world, r) for r in range(world)]
    assert parts[0][0] == 0 and parts[-1][1] == n
    assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
    sizes = [b - a for a, b in parts]
    assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)


def test_shard_range_rejects_bad_rank():
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)
    with pytest.raises(ValueError):
        shard_range(10, 0, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    try:
        sys.path.insert(0, str(ROOT))
        sys.path.insert(0, str(ROOT / "oracle"))
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        import torch
        import torch.distributed as dist
        import oracle as O
        from pbrt_rust_gb300 import generators as G
        from pbrt_rust_gb300.scene import SceneDescription, default_num_tasks
        from pbrt_rust_gb300.shard import gather_rows, shard_range, sum_images, task_range
        dist.init_process_group("gloo", rank=rank, world_size=world)

        # ray batch: each rank traces its range, the hits are gathered
        prims, rays = G.ray_soup(512, 3001, seed=3)
        lo, hi = shard_range(len(rays), world, rank)
        ob = O.OracleBVH(prims, 4, "sah")
        local = torch.from_numpy(ob.intersect(rays[lo:hi]).view(np.int32).reshape(-1, 4).copy())
        hits = gather_rows(local, len(rays)).numpy()
        full_hits = ob.intersect(rays).view(np.int32).reshape(-1, 4)

        # frame: each rank renders its tasks, the images are summed
        prims, lights, cam, smp = G.c1_scene(res=40)
        nt = default_num_tasks(40, 40)
        t0, t1 = task_range(nt, world, rank)
        desc = SceneDescription(prims, lights, 4, "sah")
        part = O.render(desc, cam, smp, nt, task_lo=t0, task_hi=t1)
        img = sum_images(torch.from_numpy(part.copy())).numpy()
        full = O.render(desc, cam, smp, nt)
        q.put((rank, bool(np.array_equal(hits, full_hits)), bool(np.array_equal(img.view(np.uint32),
                                                                               full.view(np.uint32))),
               float(full.max()), t1 - t0))
        dist.destroy_process_group()
    except Exception as e:  # reported to the parent
        q.put((rank, repr(e)))


@pytest.mark.timeout(300)
def test_two_rank_shards_merge_to_the_unsharded_result(oracle):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    for r in results:
        assert len(r) == 5, r
        rank, hits_ok, img_ok, peak, ntasks = r
        assert hits_ok, f"rank {rank}: gathered hits differ from the unsharded batch"
        assert img_ok, f"rank {rank}: summed shard images differ from the unsharded frame"
        assert peak > 0.1 and ntasks >= 1
