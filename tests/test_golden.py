"""The committed golden fixtures (tests/golden/) against the CPU oracle and
the product's host-side BVH build.

The fixtures were written by tests/golden/make_golden.py from the oracle; a
change to the oracle or to the host build that moves any stored value fails
here, on the CPU, before any GPU comparison.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import make_golden as MG  # noqa: E402

from pbrt_rust_gb300.scene import SceneDescription, default_num_tasks  # noqa: E402


def load(name):
    return np.load(GOLDEN / name)


def test_soup_hits_match_golden(oracle):
    g = load("soup_closest.npz")
    prims, _ = MG.soup_inputs()
    rays = MG.as_rays(g["rays"])
    ob = oracle.OracleBVH(prims, 4, "sah")
    assert np.array_equal(MG.hits_array(ob.intersect(rays)), g["hits"])
    assert np.array_equal(ob.intersect_p(rays), g["occluded"])
    assert (g["hits"][:, 0] >= 0).sum() > 100  # the set has real hits


def test_first_hit_walk_answers_like_the_full_search(oracle):
    """The early-exit walk the oracle counts for the any-hit roofline gives
    the reference's intersect_p answers (D11) with less work."""
    g = load("soup_closest.npz")
    prims, _ = MG.soup_inputs()
    rays = MG.as_rays(g["rays"])
    ob = oracle.OracleBVH(prims, 4, "sah")
    occ, cnt = ob.first_hit_counts(rays)
    assert np.array_equal(occ, g["occluded"])
    _, full = ob.intersect_p(rays, counters=True)
    assert 0 < cnt[0] < full[0] and cnt[1] <= full[1]


def test_oracle_scene_renders_like_the_one_shot_render(oracle):
    """OracleScene (built once, rendered many times) gives oracle.render's
    image, and counts the traversal work of camera and shadow rays."""
    prims, lights, cam, smp = MG.sphere_inputs()[:4]
    nt = default_num_tasks(48, 48)
    desc = SceneDescription(prims, lights, 4, "sah")
    img, st = oracle.OracleScene(desc).render(cam, smp, nt)
    assert np.array_equal(img.view(np.uint32), load("render_c1_48.npz")["rgb"].view(np.uint32))
    assert st[0] == 48 * 48 * 4 and st[1] > 0 and st[2] > st[0] and st[5] > 0


def test_sphere_scene_hits_match_golden(oracle):
    g = load("spheres_closest.npz")
    prims = MG.sphere_inputs()[0]
    ob = oracle.OracleBVH(prims, 4, "sah")
    rays = MG.as_rays(g["rays"])
    assert np.array_equal(MG.hits_array(ob.intersect(rays)), g["hits"])
    assert np.array_equal(ob.intersect_p(rays), g["occluded"])


def test_bvh_layout_matches_golden(lib):
    """The product's host build (what the device kernels traverse) equals the
    stored reference-algorithm BVH node for node."""
    from pbrt_rust_gb300.gpu import GpuBVHAccel
    g = load("bvh_soup.npz")
    prims, _ = MG.soup_inputs()
    b = GpuBVHAccel(prims, 4, "sah")
    assert b.depth() == int(g["depth"][0])
    assert np.array_equal(b.nodes().view(np.uint8), g["nodes"].view(np.uint8))
    assert np.array_equal(b.primitive_order(), g["order"])


@pytest.mark.parametrize("name,inputs,res", [("render_c1_48.npz", lambda: MG.sphere_inputs()[:4], 48),
                                             ("render_tris_40.npz", MG.tris_inputs, 40)])
def test_render_matches_golden(oracle, name, inputs, res):
    prims, lights, cam, smp = inputs()
    img = oracle.render(SceneDescription(prims, lights, 4, "sah"), cam, smp, default_num_tasks(res, res))
    assert np.array_equal(img.view(np.uint32), load(name)["rgb"].view(np.uint32))
