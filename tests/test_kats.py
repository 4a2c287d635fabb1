"""Known-answer tests of the reference crate, ported.

Each test cites the Rust unit test whose expected values it repeats.  They
pin the CPU oracle (and, for the BVH topology, the product's host-side
build through the C ABI, which runs without a GPU) to the reference.
"""
import ctypes as C
import math

import numpy as np
import pytest

from pbrt_rust_gb300 import abi
from pbrt_rust_gb300.scene import Primitive, Shape
from pbrt_rust_gb300.transform import Transform, mat_inverse

F = np.float32
FMAX = float(np.finfo(np.float32).max)


def ray(o, d, mint=0.0, maxt=FMAX):
    r = np.zeros(1, dtype=abi.RAY_DTYPE)
    r["o"] = o
    r["d"] = d
    r["tmin"] = mint
    r["tmax"] = maxt
    return r


def ptr(a):
    return C.c_void_p(a.ctypes.data)


# ------------------------------------------------------------------ bbox ----
def bbox_hit(oracle, lo, hi, r):
    lib = oracle.load()
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    out = np.zeros(2, np.float32)
    ok = lib.oracle_bbox_intersect(ptr(lo), ptr(hi), ptr(r), ptr(out))
    return (float(out[0]), float(out[1])) if ok else None


def test_bbox_slab_kats(oracle):
    """src/bbox.rs:553-615"""
    lo, hi = (-1, -1, -1), (1, 1, 1)
    cases = [((2, 0, 0), (-1, 0, 0), (1.0, 3.0)), ((-2, 0, 0), (1, 0, 0), (1.0, 3.0)),
             ((2, 0, 0), (1, 0, 0), None), ((-2, 0, 0), (-1, 0, 0), None),
             ((0, 2, 0), (0, -1, 0), (1.0, 3.0)), ((0, -2, 0), (0, 1, 0), (1.0, 3.0)),
             ((0, 2, 0), (0, 1, 0), None), ((0, -2, 0), (0, -1, 0), None),
             ((0, 0, 2), (0, 0, -1), (1.0, 3.0)), ((0, 0, -2), (0, 0, 1), (1.0, 3.0)),
             ((0, 0, 2), (0, 0, 1), None), ((0, 0, -2), (0, 0, -1), None)]
    for o, d, want in cases:
        assert bbox_hit(oracle, lo, hi, ray(o, d)) == want, (o, d)
    n = F(1.0) / np.sqrt(F(3.0))
    t0, t1 = bbox_hit(oracle, lo, hi, ray((-1, -1, -1), (n, n, n)))
    assert t0 == 0.0 and abs(t1 - math.sqrt(12.0)) < 1e-6
    assert bbox_hit(oracle, lo, hi, ray((1.5, 0.5, 0.5), (-0.5, 0.0, 0.5))) == (1.0, 1.0)
    assert bbox_hit(oracle, lo, hi, ray((1.5, 0.5, 0.5), (-0.5, -0.5, 0.5))) == (1.0, 1.0)
    assert bbox_hit(oracle, lo, hi, ray((2, 0, 0), (-1, 0, 0), 2.0)) == (2.0, 3.0)


def test_bbox_area_and_extent(oracle):
    """src/bbox.rs:346-401"""
    lib = oracle.load()

    def m(lo, hi):
        lo = np.asarray(lo, np.float32)
        hi = np.asarray(hi, np.float32)
        a = C.c_float()
        e = C.c_int32()
        lib.oracle_bbox_metrics(ptr(lo), ptr(hi), C.byref(a), C.byref(e))
        return a.value, e.value

    empty = ((FMAX,) * 3, (-FMAX,) * 3)
    assert m((0, 0, 0), (1, 1, 1))[0] == 6.0
    assert m(*empty)[0] == 0.0
    assert m((1, 0, 0), (1, 1, 1))[0] == 2.0
    assert m((0, 0, 0), (2, 3, 4))[0] == 52.0
    assert m((0, 0, 0), (1, 1, 1))[1] == 2
    assert m(*empty)[1] == 2
    assert m((0, 0, 0), (2, 3, 4))[1] == 2
    assert m((0, 0, 0), (4, 5, 4))[1] == 1
    assert m((0, 10, 0), (4, 5, 4))[1] == 2


# ----------------------------------------------------------------- utils ----
def test_quadratic_kats(oracle):
    """src/utils/mod.rs:366-389"""
    lib = oracle.load()

    def q(a, b, c):
        t0, t1 = C.c_float(), C.c_float()
        return (t0.value, t1.value) if lib.oracle_quadratic(a, b, c, C.byref(t0), C.byref(t1)) else None

    assert q(1.0, 0.0, 1.0) is None
    assert q(-1.0, 4.0, -4.0) == (2.0, 2.0)
    assert q(1.0, 0.0, 0.0) == (0.0, 0.0)
    assert q(1.0, -2.0, 0.0) == (0.0, 2.0)
    for i in range(2, 200):
        assert q(1.0, -float(i), 0.0) == (0.0, float(i))
    s3 = F(np.sqrt(F(3.0)))
    assert q(-1.0, 8.0, -13.0) == (float(F(-s3) + F(4.0)), float(s3 + F(4.0)))
    assert q(0.0, 1.0, 1.0) is None
    assert q(0.0, 0.0, 1.75) is None


def _partition(oracle, xs):
    a = np.array(xs, dtype=np.int64)
    oracle.load().oracle_partition_by_i64(ptr(a), len(a))
    return a


def test_partition_by_kats(oracle):
    """src/utils/mod.rs:438-517"""
    for xs in ([2, 5, 6, 1, 0, 4, 3, 2, 5, 1, 3, 3, 5], [1, 0, 0, 0, -1, 0],
               [-2, -4, 2, 2, 2, 4, 4, 4, 4, 4, 4, 4], [-2, -4, 2, 2, 2, 4, 4, 4, 4, 4, 4, -5]):
        a = _partition(oracle, xs)
        mid = len(a) // 2
        assert a[:mid].max() <= a[mid:].min()
        assert sorted(a.tolist()) == sorted(xs)
    assert _partition(oracle, [1, 2]).tolist() == [1, 2]
    assert _partition(oracle, [2, 1]).tolist() == [1, 2]
    assert _partition(oracle, [1]).tolist() == [1]
    assert _partition(oracle, [3, 1, 1]).tolist() == [1, 1, 3]
    assert _partition(oracle, [3, 1, 2]).tolist() == [1, 2, 3]
    assert _partition(oracle, [3, 3, 1]).tolist() == [1, 3, 3]
    assert _partition(oracle, [2, 2, 2]).tolist() == [2, 2, 2]
    pts = np.array([1.0, -2.0, 2.0], np.float32)  # utils/mod.rs:509-517 (x coordinates)
    oracle.load().oracle_partition_by_f32(ptr(pts), 3)
    assert pts[0] == -2.0


def test_crop_window_kats(oracle):
    """src/utils/mod.rs:519-530"""
    lib = oracle.load()

    def cw(num, count, aspect):
        o = np.zeros(4, np.float32)
        lib.oracle_crop_window(num, count, aspect, ptr(o))
        return tuple(o.tolist())

    assert cw(0, 2, 2.0) == (0.0, 0.5, 0.0, 1.0)
    assert cw(1, 2, 2.0) == (0.5, 1.0, 0.0, 1.0)
    assert cw(0, 2, 0.5) == (0.0, 1.0, 0.0, 0.5)
    assert cw(1, 2, 0.5) == (0.0, 1.0, 0.5, 1.0)
    assert cw(0, 4, 1.0) == (0.0, 0.5, 0.0, 0.5)
    assert cw(1, 4, 1.0) == (0.5, 1.0, 0.0, 0.5)
    assert cw(2, 4, 1.0) == (0.0, 0.5, 0.5, 1.0)
    assert cw(3, 4, 1.0) == (0.5, 1.0, 0.5, 1.0)


def test_sub_window_kats(oracle):
    """src/sampler/base.rs:68-89"""
    lib = oracle.load()

    def sw(xs, xe, ys, ye, num, count):
        o = np.zeros(4, np.int32)
        lib.oracle_sub_window(xs, xe, ys, ye, num, count, ptr(o))
        return tuple(o.tolist())

    assert sw(0, 10, 0, 2, 0, 20) == (0, 1, 0, 1)
    assert sw(0, 10, 0, 2, 9, 20) == (9, 10, 0, 1)
    assert sw(0, 10, 0, 2, 10, 20) == (0, 1, 1, 2)
    assert sw(0, 10, 0, 2, 19, 20) == (9, 10, 1, 2)
    assert sw(0, 10, 0, 2, 4, 5) == (8, 10, 0, 2)
    assert sw(0, 10, 0, 2, 0, 1) == (0, 10, 0, 2)
    assert sw(0, 2, 0, 10, 0, 20) == (0, 1, 0, 1)
    assert sw(0, 2, 0, 10, 9, 20) == (1, 2, 4, 5)
    assert sw(0, 2, 0, 10, 10, 20) == (0, 1, 5, 6)
    assert sw(0, 2, 0, 10, 19, 20) == (1, 2, 9, 10)
    assert sw(0, 2, 0, 10, 4, 5) == (0, 2, 8, 10)
    assert sw(0, 2, 0, 10, 0, 1) == (0, 2, 0, 10)


# ------------------------------------------------------------ sampling ----
def test_stratified_kats(oracle):
    """src/montecarlo.rs:193-249"""
    lib = oracle.load()
    calls = np.array([[1, 4, 0, 0], [1, 4, 0, 1]], np.int32)
    out = np.zeros(8, np.float32)
    lib.oracle_stratified(0, ptr(calls), 2, ptr(out))
    assert out[:4].tolist() == [0.5 / 4, 1.5 / 4, 2.5 / 4, 3.5 / 4]
    for i in range(4):
        assert i / 4 <= out[4 + i] <= (i + 1) / 4
    calls = np.array([[2, 2, 2, 0], [2, 3, 2, 1]], np.int32)
    out = np.zeros(8 + 12, np.float32)
    lib.oracle_stratified(0, ptr(calls), 2, ptr(out))
    assert out[:8].tolist() == [0.25, 0.25, 0.75, 0.25, 0.25, 0.75, 0.75, 0.75]
    j = out[8:]
    for k in range(6):
        x, y = k % 3, k // 3
        assert x / 3 <= j[2 * k] <= (x + 1) / 3
        assert y / 2 <= j[2 * k + 1] <= (y + 1) / 2


def test_rng_shuffle_properties(oracle):
    """src/rng.rs:49-87 (the only value-dependent checks on the stream)."""
    lib = oracle.load()
    one = np.array([0], np.int64)
    lib.oracle_rng_shuffle_i64(12, ptr(one), 1, 1, 0)
    assert one.tolist() == [0]
    xs = np.array([0] + [1] * 10, np.int64)
    lib.oracle_rng_shuffle_i64(12, ptr(xs), 11, 1, 1)  # after the one draw above
    assert xs[0] == 1 and sorted(xs.tolist()) == [0] + [1] * 10
    perm = np.zeros(11, np.uint64)
    lib.oracle_rng_permutation(120, ptr(perm), 11)
    assert perm[0] != 0 and sorted(perm.tolist()) == list(range(11))


def test_rng_stream_consistency(oracle):
    """random_float / random_uint are (u32 >> 8) * 2^-24 and two words, low
    first (rng.rs:15-21), read from one word stream."""
    lib = oracle.load()
    w = np.zeros(40, np.uint32)
    lib.oracle_rng_words(7, 0, 40, ptr(w))
    f = np.zeros(40, np.float32)
    lib.oracle_rng_floats(7, 40, ptr(f))
    assert np.array_equal(f, (w >> 8).astype(np.float32) * np.float32(2.0 ** -24))
    u = np.zeros(20, np.uint64)
    lib.oracle_rng_uints(7, 20, ptr(u))
    assert np.array_equal(u, w[0::2].astype(np.uint64) | (w[1::2].astype(np.uint64) << np.uint64(32)))
    w2 = np.zeros(9, np.uint32)
    lib.oracle_rng_words(7, 31, 9, ptr(w2))  # seeking across a block boundary
    assert np.array_equal(w2, w[31:40])


# ------------------------------------------------------------- filters ----
def test_filter_kats(oracle):
    """src/filter.rs:136-211"""
    ev = oracle.load().oracle_filter_eval
    for x in [0.0, 1.0, -1.0, 16.0, 0.001]:
        for y in [2.0, 0.0, -0.01, math.pi]:
            assert ev(0, 1.0, 1.0, 0, 0, x, y) == 1.0
    tri = lambda x, y: ev(1, 2.0, 2.0, 0, 0, x, y)  # noqa: E731
    assert tri(1.0, 0.0) == 0.5 and tri(0.0, 0.0) == 1.0 and tri(1.0, 1.0) == 0.25 and tri(0.5, 0.5) == 0.5625
    for x, y in [(20, 0), (-20, 0), (0, 20), (0, -20), (2, 0), (0, -2)]:
        assert tri(x, y) == 0.0
        assert ev(2, 2.0, 2.0, 1.0, 0, x, y) == 0.0
        assert ev(4, 2.0, 2.0, 1.0, 0, x, y) == 0.0
        assert ev(3, 2.0, 2.0, 0.2, 0.4, x, y) == 0.0
    g = lambda x, y: ev(2, 2.0, 2.0, 1.0, 0, x, y)  # noqa: E731
    assert g(1, 1) > 0 and g(0.5, 0) > 0 and g(1, -0.5) > 0 and g(-1, -1.5) > 0 and g(0, 0) > 0.9
    assert ev(4, 2.0, 2.0, 1.0, 0, 0, 0) > 0.9
    assert ev(3, 2.0, 2.0, 0.2, 0.4, 0, 0) > 0.8


# -------------------------------------------------------- film extents ----
def test_film_extent_kats(oracle):
    """src/camera/film.rs:362-408"""
    lib = oracle.load()
    ot, tt = float(F(1.0) / F(3.0)), float(F(2.0) / F(3.0))

    def ext(crop):
        c = np.array(crop, np.float32)
        se = np.zeros(4, np.int32)
        pe = np.zeros(4, np.int32)
        lib.oracle_film_extents(142, 12, ptr(c), 3.0, 3.0, ptr(se), ptr(pe))
        return tuple(se.tolist()), tuple(pe.tolist())

    assert ext([ot, tt, ot, tt]) == ((45, 98, 1, 11), (48, 95, 4, 8))
    assert ext([0.0, ot, ot, tt]) == ((-3, 51, 1, 11), (0, 48, 4, 8))


def test_film_extent_product_matches(lib):
    """The product's film extent (pbrtgpu_film_pixel_extent) on the same
    KAT (film.rs:392-408)."""
    from pbrt_rust_gb300.scene import Camera, Film, Filter
    ot, tt = float(F(1.0) / F(3.0)), float(F(2.0) / F(3.0))
    for crop, want in [((ot, tt, ot, tt), (48, 95, 4, 8)), ((0.0, ot, ot, tt), (0, 48, 4, 8))]:
        film = Film.image(142, 12, Filter.mean(3.0, 3.0), crop)
        cam = Camera.perspective(Transform(), (-1, 1, -1, 1), 0, 1, 0, 1, 60, film)
        e = (C.c_int32 * 4)()
        ca = cam.to_abi()
        abi.check(lib.pbrtgpu_film_pixel_extent(C.byref(ca), e))
        assert tuple(e[:]) == want
        assert film.pixel_extent() == want


# --------------------------------------------------------- transforms ----
def _xf_vec(oracle, t: Transform, v):
    out = np.zeros(3, np.float32)
    src = np.array(v, np.float32)
    ta = t.to_abi()
    oracle.load().oracle_transform_vector(C.byref(ta), ptr(src), ptr(out))
    return out


def _xf_pt(oracle, t: Transform, p):
    out = np.zeros(3, np.float32)
    src = np.array(p, np.float32)
    ta = t.to_abi()
    oracle.load().oracle_transform_point(C.byref(ta), ptr(src), ptr(out))
    return out


def _look_at(oracle, pos, look, up):
    t = abi.PbrtTransform()
    a, b, c = (np.array(pos, np.float32), np.array(look, np.float32), np.array(up, np.float32))
    oracle.load().oracle_look_at(ptr(a), ptr(b), ptr(c), C.byref(t))
    return Transform(np.array(t.m[:], np.float32), np.array(t.m_inv[:], np.float32))


def test_look_at_kats(oracle):
    """src/transform/transform.rs:526-562 (and the Python host mirror)."""
    for t in (_look_at(oracle, (1, 1, 1), (0, 0, 0), (0, 1, 0)),
              Transform.look_at((1, 1, 1), (0, 0, 0), (0, 1, 0))):
        p = _xf_pt(oracle, t, (0, 0, 0))
        assert abs(p[0]) < 1e-6 and abs(p[1]) < 1e-6 and p[2] > 1.0
        p = _xf_pt(oracle, t, (-1, -1, -1))
        assert abs(p[0]) < 1e-6 and abs(p[1]) < 1e-6 and p[2] > 2.0
    for t2 in (_look_at(oracle, (1, 2, 3), (-1, 0, 4), (0, 1, 0)),
               Transform.look_at((1, 2, 3), (-1, 0, 4), (0, 1, 0))):
        p = _xf_pt(oracle, t2, (0, 0, -3))
        assert p[2] == 0.0 and abs(p[0]) > 0.1 and abs(p[1]) > 0.1
        p = _xf_pt(oracle, t2, (0, 1, 3.5))
        assert p[2] > 1.0 and abs(p[0]) < 1e-6 and abs(p[1]) < 1e-6
    a = _look_at(oracle, (0, 1.5, -6), (0, 0, 0), (0, 1, 0))
    b = Transform.look_at((0, 1.5, -6), (0, 0, 0), (0, 1, 0))
    assert np.array_equal(a.m, b.m) and np.array_equal(a.m_inv, b.m_inv)


def test_ray_transform_kat(oracle):
    """src/transform/transform.rs:599-632"""
    rot = Transform(np.array([[0, 0, 1, 0], [0, 1, 0, 0], [-1, 0, 0, 0], [0, 0, 0, 1]], np.float32))
    # rotate_y(90) from sin/cos of 90 degrees in f32
    s = F(np.sin(F(F(90.0) * F(np.pi)) / F(180.0)))
    c = F(np.cos(F(F(90.0) * F(np.pi)) / F(180.0)))
    m = np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1]], np.float32)
    rot = Transform(m, m.T.copy())
    xf = Transform.translate((1, 1, 1)) * rot
    o = _xf_pt(oracle, xf, (0, 0, 0))
    d = _xf_vec(oracle, xf, (1, 0, 0))
    assert o.tolist() == [1.0, 1.0, 1.0]
    assert float(np.sum((d - np.array([0, 0, -1], np.float32)) ** 2)) < 1e-6


def test_matrix_inverse_kat(oracle):
    """src/transform/transform.rs:437-449 and the Python host mirror of the
    LU inverse (matrix4x4.rs:66-160) agree bit for bit."""
    m = np.array([[2, 3, 1, 5], [1, 0, 3, 1], [0, 2, -3, 2], [0, 2, 3, 1]], np.float32)
    out = np.zeros(16, np.float32)
    flat = m.reshape(-1).copy()
    assert oracle.load().oracle_matrix_invert(ptr(flat), ptr(out)) == 1
    inv = out.reshape(4, 4)
    assert np.array_equal(inv, mat_inverse(m))
    t = Transform(m, inv)
    p = _xf_pt(oracle, t.inverse(), _xf_pt(oracle, t, (1, 2, 3)))
    assert float(np.sum((p - np.array([1, 2, 3], np.float32)) ** 2)) < 1e-6


def _projection(oracle, proj: Transform, screen, xres=640, yres=480):
    out = (abi.PbrtTransform * 4)()
    sw = np.array(screen, np.float32)
    pa = proj.to_abi()
    oracle.load().oracle_projection(xres, yres, C.byref(pa), ptr(sw), out)
    return [Transform(np.array(o.m[:], np.float32), np.array(o.m_inv[:], np.float32)) for o in out]


def test_projection_kats(oracle):
    """src/camera/projective.rs:119-250"""
    ortho = Transform.translate((0.0, 0.0, -1.0))
    full = (0.0, 640.0, 0.0, 480.0)
    flip = Transform.from_matrix([[1, 0, 0, 0], [0, -1, 0, 480], [0, 0, 1, 0], [0, 0, 0, 1]])
    for proj in (ortho, Transform(),
                 Transform.from_matrix([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 2, -2], [0, 0, 1, 0]])):
        c2s, r2s, s2r, _ = _projection(oracle, proj, full)
        assert c2s == proj
    for proj in (ortho, Transform()):
        _, r2s, s2r, _ = _projection(oracle, proj, full)
        assert r2s == flip
        assert s2r == flip.inverse()
    _, r2s, s2r, _ = _projection(oracle, Transform(), (0.0, 1.0, 0.0, 1.0))
    want = Transform.from_matrix([[1 / 640, 0, 0, 0], [0, -1 / 480, 0, 1], [0, 0, 1, 0], [0, 0, 0, 1]])
    assert np.max(np.abs(r2s.m - want.m)) < 5e-5 and np.max(np.abs(r2s.m_inv - want.m_inv)) < 5e-5
    assert np.max(np.abs(s2r.m - want.m_inv)) < 5e-5 and np.max(np.abs(s2r.m_inv - want.m)) < 5e-5
    r2c = _projection(oracle, ortho, (0.0, 1.0, 0.0, 1.0))[3]
    assert _xf_vec(oracle, r2c, (160, 120, 1)).tolist() == [0.25, -0.25, 1.0]
    assert float(np.sum((_xf_vec(oracle, r2c, (480, 360, 0)) - np.array([0.75, -0.75, 0])) ** 2)) < 1e-5
    r2c = _projection(oracle, ortho, (-1.0, 1.0, -1.0, 1.0))[3]
    assert _xf_vec(oracle, r2c, (160, 120, 1)).tolist() == [0.5, -0.5, 1.0]
    assert float(np.sum((_xf_vec(oracle, r2c, (480, 360, 0)) - np.array([1.5, -1.5, 0])) ** 2)) < 1e-5


# ---------------------------------------------------------------- shapes ----
TET_PTS = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
TET_TRIS = np.array([0, 3, 2, 0, 1, 2, 0, 3, 1, 1, 2, 3], np.uint32)


def test_refine_order_kat(oracle):
    """src/shape/mesh.rs:424-436 + primitive/mod.rs:47-63: refine() yields
    tris[3].v == [2,3,0], tris[2].v == [2,1,0], tris[1].v == [1,3,0],
    tris[0].v == [3,2,1], and full refinement pops them back into index
    order, so refined primitive k is refine()'s tris[3 - k]."""
    mesh = Shape.triangle_mesh(Transform(), None, False, TET_TRIS, TET_PTS)
    bvh = oracle.OracleBVH([mesh], 1, "sah")
    refine_v = {3: [2, 3, 0], 2: [2, 1, 0], 1: [1, 3, 0], 0: [3, 2, 1]}
    for k in range(4):
        assert np.array_equal(bvh.triangle(k), TET_PTS[refine_v[3 - k]])


def _tri_hit(oracle, tri, r):
    out = np.zeros(3, np.float32)
    t = np.ascontiguousarray(tri, np.float32).reshape(-1)
    return bool(oracle.load().oracle_triangle_intersect(ptr(t), ptr(r), ptr(out)))


def test_triangle_intersect_kats(oracle):
    """src/shape/mesh.rs:477-497 on refine()'s tris[0] (v = [3, 2, 1])."""
    tri = TET_PTS[[3, 2, 1]]
    assert _tri_hit(oracle, tri, ray((0, 0, 0), (1, 1, 1)))
    assert not _tri_hit(oracle, tri, ray((1.5, 1.5, 1.5), (1, 1, 1)))
    assert _tri_hit(oracle, tri, ray((1.5, 1.5, 1.5), (-1, -1, -1)))
    assert not _tri_hit(oracle, tri, ray((1, 1, -1), (-1, -1, 1)))


def _sphere(oracle, o2w: Transform, r, z0, z1, pm, rr, mode=0):
    out = np.zeros(16, np.float32)
    ta = o2w.to_abi()
    ok = oracle.load().oracle_sphere_intersect(C.byref(ta), r, z0, z1, pm, ptr(rr), mode, ptr(out))
    return out if ok else None


def test_sphere_intersect_kats(oracle):
    """src/shape/sphere.rs:209-264"""
    xf = Transform.translate((1.0, 2.0, 1.0))
    hit = lambda d: _sphere(oracle, xf, 1.0, -1.0, 1.0, 360.0, ray((0, 0, 0), d)) is not None  # noqa: E731
    assert hit((1.0, 1.5, 1.0)) and hit((1.0, 1.0, 1.0)) and not hit((1.0, 0.5, 1.0))
    assert hit((0.0, 2.0, 1.0)) and hit((1.0, 2.0, 0.0))
    xf2 = Transform.translate((0.0, -3.0, 0.0)) * Transform.scale(2.0, 2.0, 2.0)
    down = ray((0, 0, 0), (0, -1, 0))
    assert _sphere(oracle, xf2, 0.75, -0.75, -0.5, 180.0, down) is None
    assert _sphere(oracle, xf2, 0.75, 0.5, 0.75, 180.0, down) is None
    assert _sphere(oracle, xf2, 0.75, -0.5, 0.75, 180.0, down, mode=1) is not None
    assert _sphere(oracle, xf2, 0.75, -0.5, 0.75, 180.0, ray((0, -3, 0), (0, -1, 0))) is None
    assert _sphere(oracle, xf2, 0.75, -0.5, 0.75, 180.0, ray((0, -3, 0), (0, 1, 0))) is not None
    assert _sphere(oracle, xf2, 0.75, -0.5, 0.75, 180.0, ray((0, -4, 10), (0, 0, -1))) is None


def test_sphere_dg_kat(oracle):
    """src/shape/sphere.rs:266-293"""
    xf = Transform.translate((0.0, -1.0, 0.0))
    o = _sphere(oracle, xf, 0.5, -0.5, 0.5, 360.0, ray((0, 0, 0), (0, -1, 0)), mode=1)
    t, eps, p, nn, u, v, dpdu, dpdv = o[0], o[1], o[2:5], o[5:8], o[8], o[9], o[10:13], o[13:16]
    assert t == 0.5 and eps == F(0.5) * F(5e-4)
    assert p.tolist() == [0.0, -0.5, 0.0]
    assert nn[0] == 0.0 and abs(nn[1] - 1.0) < 1e-6 and nn[2] == 0.0
    assert u == 0.25 and abs(v - 0.5) < 1e-6
    assert abs(dpdu[0] + math.pi) < 1e-6 and dpdu[1] == 0.0 and dpdu[2] == 0.0
    assert dpdv[0] == 0.0 and dpdv[1] == 0.0 and abs(dpdv[2] - math.pi / 2) < 1e-6


def _quad(oracle, kind, o2w: Transform, a, b, c, pm, rr, mode=0):
    out = np.zeros(16, np.float32)
    ta = o2w.to_abi()
    ok = oracle.load().oracle_quadric_intersect(kind, C.byref(ta), a, b, c, pm, ptr(rr), mode, ptr(out))
    return out if ok else None


def test_disk_intersect_kats(oracle):
    """src/shape/disk.rs:187-240 (height, radius, inner radius, phi max)."""
    from pbrt_rust_gb300 import abi
    D, I = abi.SHAPE_DISK, Transform()
    down = (0.0, 0.0, -1.0)
    hit = lambda xf, h, r, ri, pm, o, d=down: _quad(oracle, D, xf, h, r, ri, pm, ray(o, d)) is not None  # noqa
    assert hit(I, 0.0, 1.0, 0.0, 360.0, (0, 0, 1))
    assert not hit(I, 0.0, 1.0, 0.0, 360.0, (2, 2, 1))
    assert not hit(I, 0.0, 1.0, 0.5, 360.0, (0, 0, 1))  # through the hole
    assert not hit(I, 2.0, 1.0, 0.0, 360.0, (0, 0, 1))  # starting behind it
    assert hit(I, 0.0, 0.75, 0.25, 180.0, (0, 0.5, 1))  # top half of a half pipe
    assert not hit(I, 0.0, 0.75, 0.25, 180.0, (0, -0.5, 1))
    rz = Transform.rotate(180.0, (0.0, 0.0, 1.0))
    assert not hit(rz, 0.0, 0.75, 0.25, 180.0, (0, 0.5, 1))
    assert hit(rz, 0.0, 0.75, 0.25, 180.0, (0, -0.5, 1))
    assert not hit(rz, 0.0, 0.75, 0.25, 180.0, (1.0, 10.5, 140.0), (-1.0, -10.5, -140.0))


def test_disk_dg_kats(oracle):
    """src/shape/disk.rs:242-276."""
    from pbrt_rust_gb300 import abi
    o = _quad(oracle, abi.SHAPE_DISK, Transform(), 0.0, 1.0, 0.0, 360.0, ray((0, 0, 1), (0, 0, -1)), mode=1)
    assert o[0] == 1.0 and o[1] == F(5e-4)
    assert o[2:5].tolist() == [0.0, 0.0, 0.0] and o[5:8].tolist() == [0.0, 0.0, 1.0]
    o = _quad(oracle, abi.SHAPE_DISK, Transform(), 0.0, 0.75, 0.25, 180.0, ray((0, 0.5, 1), (0, 0, -1)), mode=1)
    assert o[0] == 1.0 and o[1] == F(5e-4)
    assert o[2:5].tolist() == [0.0, 0.5, 0.0] and o[5:8].tolist() == [0.0, 0.0, 1.0]
    assert o[8] == 0.5 and o[9] == 0.5


def test_cylinder_intersect_kats(oracle):
    """src/shape/cylinder.rs:222-296 (radius, z0, z1, phi max)."""
    from pbrt_rust_gb300 import abi
    Y, I = abi.SHAPE_CYLINDER, Transform()
    hit = lambda xf, r, z0, z1, pm, o, d: _quad(oracle, Y, xf, r, z0, z1, pm, ray(o, d)) is not None  # noqa
    assert hit(I, 0.5, -1.0, 1.0, 360.0, (1, 1, 1), (-1, -1, -1))
    assert not hit(I, 0.5, -1.0, 1.0, 360.0, (1, 1, 1), (0, 0, -1))
    assert not hit(I, 0.5, -1.0, 1.0, 360.0, (1, 1, 2), (-1, -1, 0))
    assert not hit(I, 0.5, -1.0, 1.0, 360.0, (-1, 1, -2), (1, -1, 0))
    assert not hit(I, 0.5, -1.0, 1.0, 360.0, (0.1, 0.1, -2), (0, 0, 1))  # down the middle
    assert hit(I, 0.5, -1.0, 1.0, 360.0, (0.1, 0.1, -2), (-0.4, -0.4, 1.5))  # from the inside
    xf = Transform.translate((1.0, 2.0, 3.0))
    assert hit(xf, 1.0, -3.0, 0.0, 90.0, (2, 4, 1.5), (-1, -1, 0))
    assert not hit(xf, 1.0, -3.0, 0.0, 90.0, (1, 2, 1.5), (-1, -1, 0))
    assert hit(xf, 1.0, -3.0, 0.0, 90.0, (1, 2, 1.5), (1, 1, 0))
    assert not hit(xf, 1.0, -3.0, 0.0, 90.0, (2.5, 2.5, 10), (-1, -1, -10))  # barely misses
    for pm in (360.0, 0.1, 0.0, -1.0):  # no radius, any phi max
        assert hit(I, 0.0, -1.0, 1.0, pm, (1, 1, -0.5), (-1, -1, 0))
    assert hit(I, 0.0, 0.0, 0.0, 360.0, (1, 1, 1), (-1, -1, -1))
    assert not hit(I, 0.0, -1.0, -1.0, 360.0, (1, 1, 1), (-1, -1, -1))


def test_cylinder_dg_kat(oracle):
    """src/shape/cylinder.rs:298-327."""
    from pbrt_rust_gb300 import abi
    xf = Transform.rotate(90.0, (0.0, 1.0, 0.0))
    d = np.array([0.0, -1.0, -1.0], np.float32)
    d = d * (F(1.0) / np.sqrt(F(d @ d)))
    o = _quad(oracle, abi.SHAPE_CYLINDER, xf, 1.0, -1.0, 1.0, 180.0, ray((0, 1, 1), tuple(d)), mode=1)
    t = math.sqrt(2.0) - 1.0
    assert abs(o[0] - t) < 1e-6 and abs(o[1] - t * 5e-4) < 1e-6
    s2 = math.sqrt(2.0) * 0.5
    assert np.sum((o[2:5] - [0.0, s2, s2]) ** 2) < 1e-6
    assert np.sum((o[5:8] - np.array([0.0, 1.0, 1.0]) / math.sqrt(2.0)) ** 2) < 1e-6
    assert o[8] == 0.75 and abs(o[9] - 0.5) < 1e-6
    assert np.sum((o[10:13] - [0.0, -math.pi * s2, math.pi * s2]) ** 2) < 1e-6
    assert np.sum((o[13:16] - [2.0, 0.0, 0.0]) ** 2) < 1e-6


# ------------------------------------------------------------------- BVH ----
def sphere_at(v):
    """src/primitive/aggregates/mod.rs:76-80"""
    t = Transform.translate(v)
    return Primitive.simple(Shape.sphere(t, Transform.translate(tuple(-c for c in v)), False, 1.0, -1.0, 1.0, 360.0))


def get_spheres():
    """src/primitive/aggregates/mod.rs:82-91"""
    return [sphere_at(v) for v in [(0, 0, 0), (2, 0, 0), (0, 2, 0), (2, 2, 0), (0, 0, 2), (2, 0, 2), (0, 2, 2),
                                   (2, 2, 2)]]


def both_bvhs(oracle, prims, mp, sm):
    from pbrt_rust_gb300.gpu import GpuBVHAccel
    return oracle.OracleBVH(prims, mp, sm), GpuBVHAccel(prims, mp, sm)


@pytest.mark.parametrize("sm", ["sah", "middle", "equal"])
def test_bvh_leaves_cover_prims(oracle, lib, sm):
    """src/primitive/aggregates/bvh.rs:438-455"""
    for b in both_bvhs(oracle, get_spheres(), 1, sm):
        nodes = b.nodes()
        leaves = nodes[nodes["is_leaf"] == 1]
        assert np.all(leaves["count"] == 1)
        assert sorted(leaves["offset"].tolist()) == list(range(8))
        assert b.num_primitives() == 8


@pytest.mark.parametrize("sm,idx,want", [
    ("middle", [0, 1, 4], [((-5, -1, -1), (9, 1, 1)), ((-5, -1, -1), (-1, 1, 1)), ((1, -1, -1), (9, 1, 1))]),
    ("equal", [0, 1, 6], [((-5, -1, -1), (9, 1, 1)), ((-5, -1, -1), (3, 1, 1)), ((3, -1, -1), (9, 1, 1))]),
])
def test_bvh_topology_line_kats(oracle, lib, sm, idx, want):
    """src/primitive/aggregates/bvh.rs:490-534"""
    prims = [sphere_at((x, 0, 0)) for x in (-4, -2, 2, 4, 6, 8)]
    for b in both_bvhs(oracle, prims, 1, sm):
        nodes = b.nodes()
        for i, (lo, hi) in zip(idx, want):
            assert nodes[i]["lo"].tolist() == list(map(float, lo)) and nodes[i]["hi"].tolist() == list(map(float, hi))


def test_bvh_topology_sah_kat(oracle, lib):
    """src/primitive/aggregates/bvh.rs:536-559"""
    prims = [sphere_at(v) for v in [(-2, 2, 0), (-4, 0, 0), (2, 0, 0), (4, 2, -3), (4, 1.5, -1.5), (4, 1.5, 1.5),
                                    (4, 2, 3), (4, 0, 0)]]
    want = {0: ((-5, -1, -4), (5, 3, 4)), 1: ((-5, -1, -1), (3, 3, 1)), 6: ((3, -1, -4), (5, 3, 4))}
    ob, gb = both_bvhs(oracle, prims, 1, "sah")
    for b in (ob, gb):
        nodes = b.nodes()
        for i, (lo, hi) in want.items():
            assert nodes[i]["lo"].tolist() == list(map(float, lo)) and nodes[i]["hi"].tolist() == list(map(float, hi))
    assert np.array_equal(ob.nodes().view(np.uint8), gb.nodes().view(np.uint8))
    assert np.array_equal(ob.primitive_order(), gb.primitive_order())


@pytest.mark.parametrize("sm", ["sah", "middle", "equal"])
def test_aggregate_intersection_kat(oracle, sm):
    """src/primitive/aggregates/mod.rs:93-138 (expected primitive ids 0, 4, 6)."""
    b = oracle.OracleBVH(get_spheres(), 1, sm)
    rays = np.concatenate([ray((0, 0, -1), (0, 0, 1)), ray((-1, 0, 2), (1, 0, 0)), ray((4, 0, 0), (-2, 1, 1))])
    hits = b.intersect(rays, nthreads=1)
    assert hits["prim"].tolist() == [0, 4, 6]


@pytest.mark.parametrize("mp,sm", [(1, "sah"), (10, "middle")])
def test_bvh_tetrahedron_kat(oracle, mp, sm):
    """src/primitive/aggregates/bvh.rs:457-488: intersect_p is true and the
    closest hit shrinks maxt to 1.0."""
    mesh = Shape.triangle_mesh(Transform(), None, False, TET_TRIS, TET_PTS)
    b = oracle.OracleBVH([mesh], mp, sm)
    r = ray((0.25, -1.0, 0.25), (0.0, 1.0, 0.0))
    assert b.intersect_p(r, nthreads=1)[0] == 1
    assert b.intersect(r, nthreads=1)["t"][0] == 1.0


def test_unknown_split_method_falls_back_to_sah(oracle, lib):
    """bvh.rs:341-349: an unknown method warns and uses SAH."""
    from pbrt_rust_gb300.gpu import GpuBVHAccel
    a = GpuBVHAccel(get_spheres(), 1, "bogus").nodes()
    b = GpuBVHAccel(get_spheres(), 1, "sah").nodes()
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
