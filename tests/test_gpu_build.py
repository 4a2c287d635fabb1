"""The BVH tree built on the device (PBRT_BUILD_ON_DEVICE) against the host
build: the same nodes (bounds, axes, offsets), primitive order and depth,
for every split method and shape mix, and the same traversal results."""
import numpy as np
import pytest

from pbrt_rust_gb300 import generators as G
from pbrt_rust_gb300.gpu import GpuBVHAccel, GpuScene
from pbrt_rust_gb300.scene import Primitive, Shape
from pbrt_rust_gb300.transform import Transform

pytestmark = pytest.mark.gpu


def same_tree(prims, mp=4, sm="sah"):
    h = GpuBVHAccel(prims, mp, sm)
    d = GpuBVHAccel(prims, mp, sm, build_on_device=True)
    assert d.depth() == h.depth()
    assert np.array_equal(d.primitive_order(), h.primitive_order())
    assert np.array_equal(d.nodes().view(np.uint8), h.nodes().view(np.uint8))
    return h, d


@pytest.mark.parametrize("n", [1, 3, 5, 200, 257, 5000, 60000])
def test_soup_trees_match(n):
    prims, _ = G.ray_soup(n, 1, seed=n)
    same_tree(prims)


@pytest.mark.parametrize("sm,mp", [("middle", 4), ("equal", 4), ("sah", 1), ("sah", 255)])
def test_split_methods_and_leaf_sizes(sm, mp):
    prims, _ = G.ray_soup(20000, 1, seed=7)
    same_tree(prims, mp, sm)


def test_heightfield_and_analytic_shapes():
    pts, idx, _ = G.heightfield_points(n_side=300)
    prims = [Primitive.simple(Shape.triangle_mesh(Transform(), None, False, idx, pts))]
    for i in range(64):
        t = Transform.translate((i * 0.2 - 6.0, 0.5, (i % 8) - 4.0))
        prims.append(Primitive.simple(Shape.sphere(t, None, False, 0.3, -0.3, 0.3, 360.0) if i % 3 == 0 else
                                      Shape.disk(t, None, False, 0.0, 0.4, 0.1, 360.0) if i % 3 == 1 else
                                      Shape.cylinder(t, None, False, 0.2, -0.2, 0.2, 270.0)))
    h, d = same_tree(prims)
    rays = G.incoherent_rays(G.PCG32(3), 1 << 16, (-9, -2, -9), (9, 2, 9))
    assert np.array_equal(h.intersect(rays).view(np.uint32), d.intersect(rays).view(np.uint32))


def test_scene_built_on_device_renders_the_same():
    prims, lights, cam, smp = G.c1_scene(res=48)
    from pbrt_rust_gb300.gpu import GpuSamplerRenderer
    r = GpuSamplerRenderer(smp, cam)
    a = r.render(GpuScene(prims, lights))
    b = r.render(GpuScene(prims, lights, build_on_device=True))
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
