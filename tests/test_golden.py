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
