"""GPU parity of closest-hit and any-hit traversal against the CPU oracle.

Tolerance: hit primitive indices bit-exact except where two hits lie within
1e-6 * t; t within 1e-5 relative of an FP64 recomputation; any-hit
booleans equal.  (The kernels repeat the reference's f32 arithmetic and
visiting order, so in practice every field is bit-identical.)
"""
import math

import numpy as np
import pytest

from pbrt_rust_gb300 import abi, generators as G
from pbrt_rust_gb300.gpu import GpuBVHAccel
from pbrt_rust_gb300.scene import Primitive, Shape
from pbrt_rust_gb300.transform import Transform

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def to_dev(rays):
    torch = _torch()
    a = np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8)
    return torch.from_numpy(a.copy()).cuda()


def dev_hits(bvh, rays):
    torch = _torch()
    out = bvh.intersect(to_dev(rays))
    torch.cuda.synchronize()
    return out.cpu().numpy().view(abi.HIT_DTYPE).reshape(-1)


def dev_any(bvh, rays):
    torch = _torch()
    out = bvh.intersect_p(to_dev(rays))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def f64_t(tri, r):
    """Moller-Trumbore in float64 for one triangle (p1, p2, p3) and ray."""
    p1, p2, p3 = (tri[i].astype(np.float64) for i in range(3))
    o = r["o"].astype(np.float64)
    d = r["d"].astype(np.float64)
    e1, e2 = p2 - p1, p3 - p1
    s1 = np.cross(d, e2)
    inv = 1.0 / np.dot(s1, e1)
    s = o - p1
    s2 = np.cross(s, e1)
    return np.dot(e2, s2) * inv


def assert_hits_match(oracle_bvh, got, want, rays, check_f64=True):
    assert got.shape == want.shape
    same_prim = got["prim"] == want["prim"]
    if not np.all(same_prim):
        bad = np.nonzero(~same_prim)[0]
        for i in bad:  # allowed only for near-ties
            assert got["prim"][i] >= 0 and want["prim"][i] >= 0, (i, got[i], want[i])
            assert abs(got["t"][i] - want["t"][i]) <= 1e-6 * abs(want["t"][i]), (i, got[i], want[i])
        assert len(bad) <= max(1, len(rays) // 100000)
    hit = want["prim"] >= 0
    ok = same_prim & hit
    np.testing.assert_array_equal(got["t"][ok], want["t"][ok])
    np.testing.assert_array_equal(got["b1"][ok], want["b1"][ok])
    np.testing.assert_array_equal(got["b2"][ok], want["b2"][ok])
    if check_f64:
        idx = np.nonzero(ok)[0]
        idx = idx[:: max(1, len(idx) // 500)]
        for i in idx:
            tri = oracle_bvh.triangle(int(got["prim"][i]))
            t64 = f64_t(tri, rays[i])
            assert abs(got["t"][i] - t64) <= 1e-5 * abs(t64), (i, got["t"][i], t64)


KERNELS = ["plain", "pt", "w4", "w4pt", "w4spec", "packet"]


@pytest.fixture(params=KERNELS)
def kernel(request):
    """Every traversal kernel must give the same, reference-exact results."""
    prev = abi.get_trace_kernel()
    abi.set_trace_kernel(request.param, 8)
    yield request.param
    abi.set_trace_kernel(*prev)


@pytest.fixture(scope="module")
def soup(oracle):
    prims, rays = G.ray_soup(4096, 1 << 20)
    gb = GpuBVHAccel(prims, 4, "sah")
    ob = oracle.OracleBVH(prims, 4, "sah")
    return prims, rays, gb, ob


def test_ray_soup_closest_hit_matches_oracle(soup, kernel):
    """4096 random triangles, 2^20 rays toward the centre (the plain ray-BVH
    query workload)."""
    prims, rays, gb, ob = soup
    assert np.array_equal(gb.nodes().view(np.uint8), ob.nodes().view(np.uint8))
    want = ob.intersect(rays)
    got = dev_hits(gb, rays)
    assert (want["prim"] >= 0).mean() > 0.3
    assert_hits_match(ob, got, want, rays)


def test_ray_soup_any_hit_matches_oracle(soup, kernel):
    prims, rays, gb, ob = soup
    np.testing.assert_array_equal(dev_any(gb, rays), ob.intersect_p(rays))


def test_host_buffers_match_device_buffers(soup, kernel):
    """The C ABI stages host buffers (numpy) through the device."""
    prims, rays, gb, ob = soup
    sub = rays[:50000]
    host = gb.intersect(sub)
    dev = dev_hits(gb, sub)
    assert np.array_equal(host.view(np.uint8), dev.view(np.uint8))
    np.testing.assert_array_equal(gb.intersect_p(sub), dev_any(gb, sub))


def test_finite_tmax_and_tmin(soup, oracle, kernel):
    """Segments (tmin > 0, finite tmax) as shadow rays use them."""
    prims, rays, gb, ob = soup
    r = rays[:200000].copy()
    rng = np.random.default_rng(3)
    r["tmin"] = rng.uniform(0.0, 2.0, len(r)).astype(np.float32)
    r["tmax"] = (r["tmin"] + rng.uniform(0.0, 3.0, len(r))).astype(np.float32)
    assert_hits_match(ob, dev_hits(gb, r), ob.intersect(r), r, check_f64=False)
    np.testing.assert_array_equal(dev_any(gb, r), ob.intersect_p(r))


def octant_sorted(rays):
    """Rays grouped by their direction signs (stable), so that whole warps
    share them - the coherent case the packet kernels walk together."""
    key = (np.signbit(rays["d"]).astype(np.int32) * np.array([1, 2, 4], np.int32)).sum(axis=1)
    return rays[np.argsort(key, kind="stable")]


def test_coherent_rays_match_oracle(soup, oracle, kernel):
    """Warps of rays with shared direction signs: camera-like bundles from
    two eye points, sorted by octant, full rays and segments."""
    prims, _, gb, ob = soup
    rng = np.random.default_rng(17)
    n = 1 << 17
    r = np.zeros(n, dtype=abi.RAY_DTYPE)
    eye = np.where(rng.uniform(size=(n, 1)) < 0.5, [0.1, 0.2, -3.0], [2.5, -0.3, 0.4]).astype(np.float32)
    tgt = rng.uniform(-0.6, 0.6, size=(n, 3)).astype(np.float32)
    d = tgt - eye
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r["o"] = eye
    r["d"] = d
    r["tmin"] = 1e-4
    r["tmax"] = np.float32(np.inf)
    r["tmax"][::7] = np.float32(2.5)  # some segments
    r = octant_sorted(r)
    want = ob.intersect(r)
    assert (want["prim"] >= 0).mean() > 0.2
    assert_hits_match(ob, dev_hits(gb, r), want, r)
    np.testing.assert_array_equal(dev_any(gb, r), ob.intersect_p(r))


@pytest.mark.parametrize("sm", ["middle", "equal"])
def test_other_split_methods(oracle, sm, kernel):
    prims, rays = G.ray_soup(2000, 1 << 16, seed=11)
    gb = GpuBVHAccel(prims, 4, sm)
    ob = oracle.OracleBVH(prims, 4, sm)
    assert np.array_equal(gb.nodes().view(np.uint8), ob.nodes().view(np.uint8))
    assert_hits_match(ob, dev_hits(gb, rays), ob.intersect(rays), rays)
    np.testing.assert_array_equal(dev_any(gb, rays), ob.intersect_p(rays))


def test_sphere_scene_matches_oracle(oracle, kernel):
    """Triangles + 64 translated spheres + the area-light quad; random rays."""
    prims, lights, cam, smp = G.c1_scene(res=64)
    gb = GpuBVHAccel(prims, 4, "sah")
    ob = oracle.OracleBVH(prims, 4, "sah")
    rng = G.PCG32(99)
    rays = G.incoherent_rays(rng, 1 << 18, (-4, 0, -4), (4, 3, 4))
    rays[: 1 << 17] = octant_sorted(rays[: 1 << 17])  # half of them in sign-coherent warps
    want = ob.intersect(rays)
    got = dev_hits(gb, rays)
    assert (want["prim"] >= 1).sum() > 1000
    assert_hits_match(ob, got, want, rays, check_f64=False)
    np.testing.assert_array_equal(dev_any(gb, rays), ob.intersect_p(rays))


def test_aggregate_kat_on_gpu(oracle, kernel):
    """src/primitive/aggregates/mod.rs:93-138 through the device path."""
    from test_kats import get_spheres, ray
    rays = np.concatenate([ray((0, 0, -1), (0, 0, 1)), ray((-1, 0, 2), (1, 0, 0)), ray((4, 0, 0), (-2, 1, 1))])
    for sm in ("sah", "middle", "equal"):
        gb = GpuBVHAccel(get_spheres(), 1, sm)
        assert dev_hits(gb, rays)["prim"].tolist() == [0, 4, 6]
        assert gb.intersect(rays)["prim"].tolist() == [0, 4, 6]


def test_tetrahedron_kat_on_gpu(kernel):
    """src/primitive/aggregates/bvh.rs:457-488 through the device path."""
    from test_kats import TET_PTS, TET_TRIS, ray
    mesh = Shape.triangle_mesh(Transform(), None, False, TET_TRIS, TET_PTS)
    for mp, sm in ((1, "sah"), (10, "middle")):
        gb = GpuBVHAccel([mesh], mp, sm)
        r = ray((0.25, -1.0, 0.25), (0.0, 1.0, 0.0))
        assert dev_any(gb, r)[0] == 1
        assert dev_hits(gb, r)["t"][0] == 1.0


def test_partial_sphere_kats_on_gpu(kernel):
    """src/shape/sphere.rs:209-264 as one-sphere aggregates on the device."""
    from test_kats import ray
    xf = Transform.translate((1.0, 2.0, 1.0))
    full = GpuBVHAccel([Shape.sphere(xf, None, False, 1.0, -1.0, 1.0, 360.0)], 1, "sah")
    dirs = [(1.0, 1.5, 1.0), (1.0, 1.0, 1.0), (1.0, 0.5, 1.0), (0.0, 2.0, 1.0), (1.0, 2.0, 0.0)]
    rays = np.concatenate([ray((0, 0, 0), d) for d in dirs])
    assert dev_any(full, rays).tolist() == [1, 1, 0, 1, 1]
    xf2 = Transform.translate((0.0, -3.0, 0.0)) * Transform.scale(2.0, 2.0, 2.0)

    def sph(z0, z1):
        return GpuBVHAccel([Shape.sphere(xf2, None, False, 0.75, z0, z1, 180.0)], 1, "sah")

    down = ray((0, 0, 0), (0, -1, 0))
    assert dev_any(sph(-0.75, -0.5), down)[0] == 0
    assert dev_any(sph(0.5, 0.75), down)[0] == 0
    s2 = sph(-0.5, 0.75)
    assert dev_hits(s2, down)["prim"][0] == 0
    assert dev_any(s2, ray((0, -3, 0), (0, -1, 0)))[0] == 0
    assert dev_any(s2, ray((0, -3, 0), (0, 1, 0)))[0] == 1
    assert dev_any(s2, ray((0, -4, 10), (0, 0, -1)))[0] == 0


def test_edge_cases(oracle, kernel):
    """Empty batches, an empty aggregate, axis-aligned and degenerate rays."""
    torch = _torch()
    from test_kats import TET_PTS, TET_TRIS, ray
    mesh = Shape.triangle_mesh(Transform(), None, False, TET_TRIS, TET_PTS)
    gb = GpuBVHAccel([mesh], 1, "sah")
    ob = oracle.OracleBVH([mesh], 1, "sah")
    empty = np.zeros(0, dtype=abi.RAY_DTYPE)
    assert gb.intersect(empty).shape == (0,)
    assert gb.intersect_p(empty).shape == (0,)
    none = GpuBVHAccel([], 4, "sah")
    r = ray((0, 0, 0), (1, 1, 1))
    assert none.intersect(r)["prim"][0] == -1 and none.intersect_p(r)[0] == 0
    lo, hi = none.world_bound()
    assert lo[0] == np.finfo(np.float32).max and hi[0] == -np.finfo(np.float32).max
    cases = [ray((0.25, -1, 0.25), (0, 1, 0)), ray((-1, 0.25, 0.25), (1, 0, 0)), ray((0.25, 0.25, -1), (0, 0, 1)),
             ray((0.25, 0.25, 5), (0, 0, -1)), ray((0, 0, 0), (0, 0, 0)), ray((0.2, 0.2, 0.2), (1, 0, 0)),
             ray((0.25, -1, 0.25), (0, 1, 0), 2.0, 1.0), ray((0.25, -1, 0.25), (-0.0, 1, -0.0)),
             ray((0, 0, 0), (1, 1, 1), 0.0, float("inf")), ray((1, 0, 0), (-1, 1, 0))]
    rays = np.concatenate(cases)
    want = ob.intersect(rays, nthreads=1)
    got = dev_hits(gb, rays)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    np.testing.assert_array_equal(dev_any(gb, rays), ob.intersect_p(rays, nthreads=1))
    assert torch.cuda.is_available()


def test_world_bound_matches_oracle(soup):
    prims, rays, gb, ob = soup
    for a, b in zip(gb.world_bound(), ob.world_bound()):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name,reorder,chunk", [("plain", True, 0), ("pt", True, 0), ("w4", True, 0),
                                                ("w4pt", True, 0), ("w4pt", True, 64), ("w4pt", False, 32),
                                                ("w4pt", False, 256)])
def test_reordered_batches_are_bit_identical(oracle, name, reorder, chunk):
    """With ray reordering on, batches of 32768+ rays are binned by direction
    and origin before traversal; with a chunk size, the persistent warps take
    rays from a shared counter.  Every hit must still equal the oracle's, at
    its own index, for host and device buffers."""
    before = abi.get_trace_config()
    abi.set_trace_config(kernel=name, reorder=reorder, chunk=chunk)
    try:
        prims, _ = G.ray_soup(4096, 1, seed=9)
        lo, hi = np.array([-1.5] * 3, np.float32), np.array([1.5] * 3, np.float32)
        rays = G.incoherent_rays(G.PCG32(77), 1 << 17, lo, hi)
        g = GpuBVHAccel(prims, 4, "sah")
        o = oracle.OracleBVH(prims, 4, "sah")
        want = o.intersect(rays)
        assert (want["prim"] >= 0).sum() > 1000
        for got in (g.intersect(rays), dev_hits(g, rays)):
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
        want_any = o.intersect_p(rays)
        assert np.array_equal(g.intersect_p(rays), want_any)
        assert np.array_equal(dev_any(g, rays), want_any)
        small = rays[:1000]  # below the reorder threshold
        assert np.array_equal(g.intersect(small).view(np.uint32), want[:1000].view(np.uint32))
    finally:
        abi.set_trace_config(**before)


def test_disks_and_cylinders_match_oracle(oracle, kernel):
    """Full disks and cylinders (no phi clip) are bit-exact; partial ones
    compare phi = atan2 against phi_max with CUDA's atan2f instead of the
    host's, which may differ in the last bit exactly at the clip edge."""
    from pbrt_rust_gb300.scene import Primitive, Shape
    prims = []
    for i in range(40):
        t = Transform.translate((((i * 37) % 11) * 0.4 - 2.0, ((i * 17) % 7) * 0.5 - 1.5, (i % 5) * 0.6 - 1.2)) \
            * Transform.rotate(23.0 * i, (0.3, 1.0, 0.2))
        full = i % 3 != 0
        pm = 360.0 if full else 90.0 + 7.0 * i
        s = (Shape.disk(t, None, i % 4 == 1, 0.05 * (i % 4), 0.35, 0.1 * (i % 2), pm) if i % 2
             else Shape.cylinder(t, None, i % 4 == 0, 0.25, -0.3, 0.3, pm))
        prims.append(Primitive.simple(s))
    rays = G.rays_toward_center(G.PCG32(8), 1 << 16, radius=6.0, target=2.0)
    g = GpuBVHAccel(prims, 4, "sah")
    o = oracle.OracleBVH(prims, 4, "sah")
    got, want = g.intersect(rays), o.intersect(rays)
    assert (want["prim"] >= 0).sum() > 5000
    same = np.all(got.view(np.uint32).reshape(-1, 4) == want.view(np.uint32).reshape(-1, 4), axis=1)
    bad = np.nonzero(~same)[0]
    assert len(bad) <= len(rays) // 10000, bad[:10]  # clip-edge ties of partial shapes only
    full_only = [p for i, p in enumerate(prims) if i % 3 != 0]
    g2, o2 = GpuBVHAccel(full_only, 4, "sah"), oracle.OracleBVH(full_only, 4, "sah")
    assert np.array_equal(g2.intersect(rays).view(np.uint32), o2.intersect(rays).view(np.uint32))
    assert np.array_equal(g2.intersect_p(rays), o2.intersect_p(rays))


def degenerate_scene_and_rays(n_tris: int = 600, seed: int = 5, nonfinite: bool = False):
    """Triangles with vertices on a 0.25 grid (rays can run exactly along box
    planes and through corners) - with `nonfinite`, some with NaN or infinite
    coordinates - and rays that start on grid planes with directions that
    have +-0, denormal, tiny or large components (with `nonfinite`, so large
    that the triangle test overflows), plus reversed [tmin, tmax] and
    infinite tmax."""
    rng = np.random.default_rng(seed)
    pts = (rng.integers(-8, 9, size=(n_tris, 3, 3)) * 0.25).astype(np.float32)
    if nonfinite:
        pts[5, 0, 0] = np.nan
        pts[6, :, 1] = np.nan
        pts[7, 1, 2] = np.inf
        pts[8, :, :] = np.nan
        pts[9, 2, 0] = -np.inf
    mesh = Shape.triangle_mesh(Transform(), None, False, np.arange(3 * n_tris, dtype=np.uint32), pts.reshape(-1, 3))
    n = 1 << 14
    r = np.zeros(n, dtype=abi.RAY_DTYPE)
    r["o"] = (rng.integers(-12, 13, size=(n, 3)) * 0.25).astype(np.float32)
    d = rng.integers(-2, 3, size=(n, 3)).astype(np.float32)
    d[d.sum(axis=1) == 0, 0] = 1.0
    huge = 3.0e38 if nonfinite else 1.0e30  # 3e38 overflows the triangle test's products to NaN
    special = np.array([0.0, -0.0, 1e-40, -1e-40, 1e-30, huge], np.float32)
    k = np.arange(n) % 3 == 0
    d[k, rng.integers(0, 3, size=n)[k]] = special[rng.integers(0, 6, size=n)[k]]
    r["d"] = d
    r["tmin"] = np.where(np.arange(n) % 17 == 0, 5.0, 0.0).astype(np.float32)
    r["tmax"] = np.where(np.arange(n) % 5 == 0, np.inf, np.where(np.arange(n) % 17 == 0, 1.0, 8.0)).astype(np.float32)
    return mesh, r


def same_hits(a, b):
    """Equal hits, a NaN equal to any NaN (device and host NaN payloads differ)."""
    if not np.array_equal(a["prim"], b["prim"]):
        return False
    return all(np.array_equal(a[f], b[f], equal_nan=True) for f in ("t", "b1", "b2"))


def test_degenerate_rays_match_oracle(oracle, kernel):
    """Both slab tests (the min/max one for rays with finite origin and 1/d,
    the literal one for the others) against the oracle on grid-aligned
    geometry.  A direction with a tiny component can overflow the triangle
    test's 1/divisor, giving a hit with NaN barycentrics as in the
    reference; NaN payloads differ between device and host."""
    mesh, rays = degenerate_scene_and_rays()
    for mp in (1, 4):
        g, o = GpuBVHAccel([mesh], mp, "sah"), oracle.OracleBVH([mesh], mp, "sah")
        want = o.intersect(rays)
        assert (want["prim"] >= 0).sum() > 2000
        assert same_hits(dev_hits(g, rays), want)
        assert np.array_equal(dev_any(g, rays), o.intersect_p(rays))


@pytest.mark.parametrize("name", ["plain", "pt", "w4", "w4pt"])
def test_nonfinite_vertices_match_oracle(oracle, name):
    """Triangles with NaN or infinite vertices and overflowing directions: a
    triangle test can accept a hit with t or barycentrics NaN (comparisons
    with NaN are false), as the reference does, after which the reference's
    box tests ignore maxt; walks that accepted a NaN distance are replayed
    in exact mode.  Equal to the oracle (NaN payloads aside).  The
    speculative-leaf kernel assumes hits lie inside their boxes and is left
    out."""
    before = abi.get_trace_config()
    abi.set_trace_config(kernel=name)
    try:
        mesh, rays = degenerate_scene_and_rays(nonfinite=True)
        g, o = GpuBVHAccel([mesh], 1, "sah"), oracle.OracleBVH([mesh], 1, "sah")
        want = o.intersect(rays)
        assert np.isnan(want["t"]).sum() > 50
        assert same_hits(dev_hits(g, rays), want)
        assert np.array_equal(dev_any(g, rays), o.intersect_p(rays))
    finally:
        abi.set_trace_config(**before)


def test_nonfinite_vertices_from_pinned_host_memory(oracle):
    """The NaN-distance case through the host-buffer forms: rays in pinned
    memory (16 copies of the degenerate set, enough for the streamed form),
    closest hits written out to pinned memory by the walk and the marked
    ones rewritten there by the exact replay; pipelined and in place too.
    Equal to the oracle (NaN payloads aside)."""
    import os
    torch = _torch()
    mesh, rays = degenerate_scene_and_rays(nonfinite=True)
    rays = np.tile(rays, 16)
    g, o = GpuBVHAccel([mesh], 1, "sah"), oracle.OracleBVH([mesh], 1, "sah")
    want, want_any = o.intersect(rays), o.intersect_p(rays)
    assert np.isnan(want["t"]).sum() > 800
    pinned = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
    saved = {k: os.environ.get(k) for k in ("PBRT_STREAM_IN", "PBRT_HOST_MAPPED")}
    try:
        for stream_in, mapped in (("1", "0"), ("0", "0"), ("1", "1")):
            os.environ["PBRT_STREAM_IN"], os.environ["PBRT_HOST_MAPPED"] = stream_in, mapped
            out = torch.full((len(rays), 4), 7.0, dtype=torch.float32).pin_memory()
            g.intersect(pinned, out=out)
            assert same_hits(out.numpy().view(abi.HIT_DTYPE).reshape(-1), want), (stream_in, mapped)
            occ = torch.full((len(rays),), 9, dtype=torch.uint8).pin_memory()
            g.intersect_p(pinned, out=occ)
            assert np.array_equal(occ.numpy(), want_any), (stream_in, mapped)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def test_pipelined_host_buffers_equal_device_buffers():
    """Host-buffer calls of 2^19+ rays run in chunks whose copies overlap
    the other chunks' traversal; every hit must land as with device
    buffers, for pageable and pinned host memory and a ray count that does
    not divide into the chunks."""
    torch = _torch()
    prims, _ = G.ray_soup(4096, 1, seed=4)
    g = GpuBVHAccel(prims, 4, "sah")
    lo, hi = np.array([-1.5] * 3, np.float32), np.array([1.5] * 3, np.float32)
    rays = G.incoherent_rays(G.PCG32(31), (1 << 20) + 12345, lo, hi)
    want, want_any = dev_hits(g, rays), dev_any(g, rays)
    assert (want["prim"] >= 0).sum() > 10000
    assert np.array_equal(g.intersect(rays).view(np.uint32), want.view(np.uint32))
    assert np.array_equal(g.intersect_p(rays), want_any)
    pinned = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
    out = torch.empty((len(rays), 4), dtype=torch.float32).pin_memory()
    g.intersect(pinned, out=out)
    assert np.array_equal(out.numpy().view(np.uint32).reshape(-1), want.view(np.uint32).reshape(-1))


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["streamed", "in_place", "pipelined"])
def test_pinned_host_buffers_every_form(monkeypatch, form):
    """Pinned host rays take the streamed form by default (the traversal
    starts at once, the rays follow in pieces it waits for), are read and
    written in place with PBRT_HOST_MAPPED=1 and go through the copy
    pipeline with PBRT_STREAM_IN=0.  Every form, with pinned, pageable and
    device outputs and a ray count that fills no whole piece, gives the
    device-buffer results bit for bit."""
    torch = _torch()
    prims, _ = G.ray_soup(4096, 1, seed=5)
    g = GpuBVHAccel(prims, 4, "sah")
    lo, hi = np.array([-1.5] * 3, np.float32), np.array([1.5] * 3, np.float32)
    rays = G.incoherent_rays(G.PCG32(37), (1 << 19) + 777, lo, hi)
    want, want_any = dev_hits(g, rays), dev_any(g, rays)
    assert (want["prim"] >= 0).sum() > 5000
    monkeypatch.setenv("PBRT_HOST_MAPPED", "1" if form == "in_place" else "0")
    monkeypatch.setenv("PBRT_STREAM_IN", "0" if form == "pipelined" else "1")
    pinned = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
    for rep in range(2):  # the second call reuses the handle's staging and flags
        out = torch.full((len(rays), 4), 7.0, dtype=torch.float32).pin_memory()
        g.intersect(pinned, out=out)
        assert np.array_equal(out.numpy().view(np.uint32).reshape(-1), want.view(np.uint32).reshape(-1)), rep
        occ = torch.full((len(rays),), 9, dtype=torch.uint8).pin_memory()
        g.intersect_p(pinned, out=occ)
        assert np.array_equal(occ.numpy(), want_any), rep
    dout = torch.full((len(rays), 4), 7.0, dtype=torch.float32, device="cuda")
    g.intersect(pinned, out=dout)
    assert np.array_equal(dout.cpu().numpy().view(np.uint32).reshape(-1), want.view(np.uint32).reshape(-1))
    docc = torch.full((len(rays),), 9, dtype=torch.uint8, device="cuda")
    g.intersect_p(pinned, out=docc)
    assert np.array_equal(docc.cpu().numpy(), want_any)
    hout = torch.full((len(rays), 4), 7.0, dtype=torch.float32).pin_memory()  # device rays, host hits
    g.intersect(to_dev(rays), out=hout)
    assert np.array_equal(hout.numpy().view(np.uint32).reshape(-1), want.view(np.uint32).reshape(-1))
    pout = torch.full((len(rays), 4), 7.0, dtype=torch.float32)  # pageable
    g.intersect(pinned, out=pout)
    assert np.array_equal(pout.numpy().view(np.uint32).reshape(-1), want.view(np.uint32).reshape(-1))
    pocc = torch.full((len(rays),), 9, dtype=torch.uint8)
    g.intersect_p(pinned, out=pocc)
    assert np.array_equal(pocc.numpy(), want_any)


@pytest.mark.gpu
def test_streamed_form_recovers_when_the_copies_come_late(monkeypatch):
    """When the ray copies do not run beside the streamed walk (as under a
    profiler that serialises work; PBRT_TEST_HOLD_STREAM_COPIES=1 queues them
    only after the walk has given up), the walk's bounded wait runs out and
    the call traces the staged rays again: same results, bounded delay."""
    import time
    torch = _torch()
    prims, _ = G.ray_soup(4096, 1, seed=8)
    g = GpuBVHAccel(prims, 4, "sah")
    lo, hi = np.array([-1.5] * 3, np.float32), np.array([1.5] * 3, np.float32)
    rays = G.incoherent_rays(G.PCG32(47), (1 << 18) + 55, lo, hi)
    want, want_any = dev_hits(g, rays), dev_any(g, rays)
    pinned = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
    monkeypatch.setenv("PBRT_TEST_HOLD_STREAM_COPIES", "1")
    out = torch.full((len(rays), 4), 7.0, dtype=torch.float32).pin_memory()
    t0 = time.perf_counter()
    g.intersect(pinned, out=out)
    assert 0.04 < time.perf_counter() - t0 < 5.0
    assert np.array_equal(out.numpy().view(np.uint32).reshape(-1), want.view(np.uint32).reshape(-1))
    occ = torch.full((len(rays),), 9, dtype=torch.uint8).pin_memory()
    g.intersect_p(pinned, out=occ)
    assert np.array_equal(occ.numpy(), want_any)
    monkeypatch.delenv("PBRT_TEST_HOLD_STREAM_COPIES")
    out.fill_(7.0)
    g.intersect(pinned, out=out)  # and the next call streams normally
    assert np.array_equal(out.numpy().view(np.uint32).reshape(-1), want.view(np.uint32).reshape(-1))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [(1 << 17) - 1, 1 << 17, (1 << 17) + 1, 3 * (1 << 16) + 5, (1 << 21) + 3])
def test_streamed_form_at_its_piece_boundaries(n):
    """Ray counts either side of the streamed form's threshold (2^17) and of
    its piece sizes (2^16 rays, more for 2^21 + 3 rays: 16 pieces of 2^17):
    pinned host rays and hits equal the device-buffer results."""
    torch = _torch()
    prims, _ = G.ray_soup(2048, 1, seed=9)
    g = GpuBVHAccel(prims, 4, "sah")
    lo, hi = np.array([-1.5] * 3, np.float32), np.array([1.5] * 3, np.float32)
    rays = G.incoherent_rays(G.PCG32(53), n, lo, hi)
    want, want_any = dev_hits(g, rays), dev_any(g, rays)
    pinned = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
    out = torch.full((n, 4), 7.0, dtype=torch.float32).pin_memory()
    g.intersect(pinned, out=out)
    assert np.array_equal(out.numpy().view(np.uint32).reshape(-1), want.view(np.uint32).reshape(-1))
    occ = torch.full((n,), 9, dtype=torch.uint8).pin_memory()
    g.intersect_p(pinned, out=occ)
    assert np.array_equal(occ.numpy(), want_any)


@pytest.mark.gpu
def test_host_buffer_calls_from_several_threads():
    """Four host threads share one handle, each with its own stream and its
    own pinned or pageable buffers: the calls serialise on the handle's
    staging buffers and flags, and every result equals the device-buffer
    one."""
    import threading
    torch = _torch()
    prims, _ = G.ray_soup(4096, 1, seed=10)
    g = GpuBVHAccel(prims, 4, "sah")
    lo, hi = np.array([-1.5] * 3, np.float32), np.array([1.5] * 3, np.float32)
    sets = [G.incoherent_rays(G.PCG32(60 + k), (1 << 18) + 17 * k, lo, hi) for k in range(4)]
    wants = [(dev_hits(g, r).view(np.uint32).reshape(-1), dev_any(g, r)) for r in sets]
    errors = []

    def work(k):
        try:
            stream = torch.cuda.Stream()
            host = torch.from_numpy(sets[k].view(np.float32).reshape(-1, 8).copy())
            if k % 2 == 0:
                host = host.pin_memory()
            for _ in range(3):
                out = torch.full((len(sets[k]), 4), 7.0, dtype=torch.float32)
                occ = torch.full((len(sets[k]),), 9, dtype=torch.uint8)
                if k % 2 == 0:
                    out, occ = out.pin_memory(), occ.pin_memory()
                g.intersect(host, out=out, stream=stream)
                g.intersect_p(host, out=occ, stream=stream)
                if not np.array_equal(out.numpy().view(np.uint32).reshape(-1), wants[k][0]):
                    errors.append(f"thread {k}: closest hits differ")
                if not np.array_equal(occ.numpy(), wants[k][1]):
                    errors.append(f"thread {k}: any hits differ")
        except Exception as e:  # reported below
            errors.append(f"thread {k}: {e!r}")

    threads = [threading.Thread(target=work, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors


def _streamed(bvh, rays_d, out_d, ready, shift, any_hit, stream):
    import ctypes as C
    lib = abi.load()
    hits = None if any_hit else C.c_void_p(out_d.data_ptr())
    occ = C.c_void_p(out_d.data_ptr()) if any_hit else None
    return lib.pbrtgpu_intersect_streamed(bvh._h, C.c_void_p(rays_d.data_ptr()), rays_d.shape[0], hits, occ,
                                          C.c_void_p(ready.data_ptr()), shift, C.c_void_p(stream.cuda_stream))


@pytest.mark.gpu
@pytest.mark.parametrize("any_hit", [False, True])
def test_streamed_rays_arriving_during_the_walk(any_hit):
    """pbrtgpu_intersect_streamed: the rays and the piece flags are copied
    on another stream that starts with the walk, so warps wait for pieces
    that are still in flight; the results equal the device-buffer call."""
    torch = _torch()
    prims, _ = G.ray_soup(4096, 1, seed=6)
    g = GpuBVHAccel(prims, 4, "sah")
    lo, hi = np.array([-1.5] * 3, np.float32), np.array([1.5] * 3, np.float32)
    n, shift = (1 << 18) + 4321, 14
    rays = G.incoherent_rays(G.PCG32(41), n, lo, hi)
    want = dev_any(g, rays) if any_hit else dev_hits(g, rays).view(np.uint32).reshape(-1, 4)
    pieces = (n + (1 << shift) - 1) >> shift
    host = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
    ones = torch.ones(pieces, dtype=torch.int32).pin_memory()
    s, side = torch.cuda.Stream(), torch.cuda.Stream()
    for rep in range(2):
        rays_d = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
        ready = torch.zeros(pieces, dtype=torch.int32, device="cuda")
        out = (torch.full((n,), 9, dtype=torch.uint8, device="cuda") if any_hit
               else torch.full((n, 4), 7.0, dtype=torch.float32, device="cuda"))
        torch.cuda.synchronize()
        start = torch.cuda.Event()
        start.record(s)
        side.wait_event(start)
        with torch.cuda.stream(side):
            for k in range(pieces):
                lo_k, hi_k = k << shift, min(n, (k + 1) << shift)
                rays_d[lo_k:hi_k].copy_(host[lo_k:hi_k], non_blocking=True)
                ready[k:k + 1].copy_(ones[k:k + 1], non_blocking=True)
        assert _streamed(g, rays_d, out, ready, shift, any_hit, s) == abi.PBRT_OK
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.array_equal(got if any_hit else got.view(np.uint32), want), rep


@pytest.mark.gpu
def test_streamed_walk_gives_up_on_pieces_that_never_arrive():
    """A piece whose flag nothing sets: the walk's bounded wait runs out,
    the call returns PBRT_ERR_TIMEOUT, the pieces that did arrive are
    traced, and the next call on the same handle works."""
    torch = _torch()
    import time
    prims, _ = G.ray_soup(4096, 1, seed=7)
    g = GpuBVHAccel(prims, 4, "sah")
    lo, hi = np.array([-1.5] * 3, np.float32), np.array([1.5] * 3, np.float32)
    n, shift = 1 << 17, 14
    rays = G.incoherent_rays(G.PCG32(43), n, lo, hi)
    want = dev_hits(g, rays).view(np.uint32).reshape(-1, 4)
    rays_d = to_dev(rays)
    ready = torch.zeros(n >> shift, dtype=torch.int32, device="cuda")
    ready[:4] = 1  # pieces 0-3 arrived, 4-7 never do
    out = torch.full((n, 4), 7.0, dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    assert _streamed(g, rays_d, out, ready, shift, False, s) == abi.PBRT_ERR_TIMEOUT
    assert 1.5 < time.perf_counter() - t0 < 30.0
    got = out.cpu().numpy().view(np.uint32)
    assert np.array_equal(got[:4 << shift], want[:4 << shift])
    ready.fill_(1)
    out.fill_(7.0)
    torch.cuda.synchronize()
    assert _streamed(g, rays_d, out, ready, shift, False, s) == abi.PBRT_OK
    assert np.array_equal(out.cpu().numpy().view(np.uint32), want)
    assert np.array_equal(dev_hits(g, rays).view(np.uint32).reshape(-1, 4), want)
