"""Seeded synthetic workloads (the reference ships no scenes or datasets).

Random numbers come from PCG32 (O'Neill 2014, XSH-RR output, the
pcg32_srandom_r seeding with a stream selector), vectorised with the
closed-form LCG jump so that large scenes generate quickly; each config's
seed is 0x9E3779B9 ^ config_index ^ (scene_index << 8).  Uniform floats
are (u32 >> 8) * 2^-24.  Geometry is computed in float64 and stored as
float32.

  ray_soup      4096 random triangles + 2^20 rays toward the centre
  c1_scene      512x512 render: ground quad, 64 matte spheres, point light,
                quad area light, 2x2 jittered strata
  heightfield   708x708-vertex terrain (999,698 triangles) + area light,
                1024x1024 at 16 spp, and 2^22 incoherent rays
  instanced_forest  two object definitions (a triangle "tree" with a sphere
                crown and a disk base; a cylinder with a mesh cap) placed by
                rotated, scaled TransformedPrimitive instances on a ground
                quad, point + area light
"""
from __future__ import annotations

import dataclasses
import functools
import math

import numpy as np

from . import abi
from .scene import (Camera, DiffuseAreaLight, Film, Filter, InstanceDefinition, MatteMaterial, PointLight,
                    Primitive, Shape, StratifiedSampler)
from .transform import Transform

_MUL = 6364136223846793005
_MASK = (1 << 64) - 1


def config_seed(config_index: int, scene_index: int = 0) -> int:
    return 0x9E3779B9 ^ config_index ^ (scene_index << 8)


class PCG32:
    """PCG32 with vectorised draws.  ``uint32(n)`` returns the next n outputs."""

    def __init__(self, seed: int, stream: int = 54):
        self.inc = ((stream << 1) | 1) & _MASK
        self.state = 0
        self._step()
        self.state = (self.state + seed) & _MASK
        self._step()

    def _step(self) -> None:
        self.state = (self.state * _MUL + self.inc) & _MASK

    @staticmethod
    @functools.lru_cache(maxsize=16)
    def _jump_tables(n: int, inc: int):
        """A^k and C_k (k = 0..n-1) with s_k = A^k s_0 + C_k (mod 2^64)."""
        a = np.empty(n, dtype=np.uint64)
        c = np.empty(n, dtype=np.uint64)
        ak, ck = 1, 0
        for k in range(n):
            a[k] = ak
            c[k] = ck
            ck = (ck * _MUL + inc) & _MASK
            ak = (ak * _MUL) & _MASK
        return a, c, ak, ck

    def uint32(self, n: int) -> np.ndarray:
        block = min(max(n, 1), 1 << 16)
        a, c, ab, cb = self._jump_tables(block, self.inc)
        out = np.empty(n, dtype=np.uint32)
        s = self.state
        pos = 0
        with np.errstate(over="ignore"):
            while pos < n:
                m = min(block, n - pos)
                st = a[:m] * np.uint64(s) + c[:m]  # states s_0 .. s_{m-1} (outputs use the old state)
                xs = (((st >> np.uint64(18)) ^ st) >> np.uint64(27)).astype(np.uint32)
                rot = (st >> np.uint64(59)).astype(np.uint32)
                out[pos:pos + m] = (xs >> rot) | (xs << ((np.uint32(32) - rot) & np.uint32(31)))
                pos += m
                s = (ab * s + cb) & _MASK if m == block else (int(a[m - 1]) * s + int(c[m - 1])) * _MUL + self.inc
                s &= _MASK
        self.state = s
        return out

    def uniform(self, n: int) -> np.ndarray:
        """n floats in [0, 1) as float64 (exact values of (u >> 8) * 2^-24)."""
        return (self.uint32(n) >> np.uint32(8)).astype(np.float64) * (1.0 / 16777216.0)


# ------------------------------------------------------------------ configs --
def random_triangle_soup(rng: PCG32, n_tris: int, extent: float = 1.0, offset: float = 0.05,
                         center=(0.0, 0.0, 0.0)) -> tuple[np.ndarray, np.ndarray]:
    """n triangles: centroid U[-extent, extent]^3, vertices = centroid +
    U[-offset, offset]^3 (12 draws per triangle, in that order)."""
    u = rng.uniform(12 * n_tris).reshape(n_tris, 12)
    cen = (u[:, 0:3] * 2.0 - 1.0) * extent + np.asarray(center, dtype=np.float64)
    off = (u[:, 3:12].reshape(n_tris, 3, 3) * 2.0 - 1.0) * offset
    pts = (cen[:, None, :] + off).reshape(-1, 3).astype(np.float32)
    idx = np.arange(3 * n_tris, dtype=np.uint32)
    return pts, idx


def rays_toward_center(rng: PCG32, n: int, radius: float = 3.0, target: float = 0.5,
                       tmin: float = 1e-4, tmax: float = math.inf) -> np.ndarray:
    """Origins uniform on a sphere of `radius`, directions normalised toward
    a point uniform in [-target, target]^3 (5 draws per ray)."""
    u = rng.uniform(5 * n).reshape(n, 5)
    z = 1.0 - 2.0 * u[:, 0]
    phi = 2.0 * math.pi * u[:, 1]
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    o = radius * np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    t = (u[:, 2:5] * 2.0 - 1.0) * target
    d = t - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(n, dtype=abi.RAY_DTYPE)
    rays["o"] = o.astype(np.float32)
    rays["d"] = d.astype(np.float32)
    rays["tmin"] = tmin
    rays["tmax"] = tmax
    return rays


def incoherent_rays(rng: PCG32, n: int, lo, hi, tmin: float = 1e-4, tmax: float = math.inf) -> np.ndarray:
    """Origins uniform in the box [lo, hi], directions uniform on the unit
    sphere (5 draws per ray)."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    u = rng.uniform(5 * n).reshape(n, 5)
    o = lo + u[:, 0:3] * (hi - lo)
    z = 1.0 - 2.0 * u[:, 3]
    phi = 2.0 * math.pi * u[:, 4]
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    d = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    rays = np.zeros(n, dtype=abi.RAY_DTYPE)
    rays["o"] = o.astype(np.float32)
    rays["d"] = d.astype(np.float32)
    rays["tmin"] = tmin
    rays["tmax"] = tmax
    return rays


def ray_soup(n_tris: int = 4096, n_rays: int = 1 << 20, seed: int | None = None):
    """Plain ray-BVH queries: random triangle soup + rays toward the centre.
    Returns (primitives, rays)."""
    rng = PCG32(config_seed(0) if seed is None else seed)
    pts, idx = random_triangle_soup(rng, n_tris)
    mesh = Shape.triangle_mesh(Transform(), None, False, idx, pts)
    rays = rays_toward_center(rng, n_rays)
    return [Primitive.geometric(mesh)], rays


def quad_light_mesh(center, size: float, facing_down: bool = True) -> Shape:
    """A horizontal square of two triangles whose geometric normal (as the
    reference computes it for refined triangles) points -y."""
    cx, cy, cz = center
    h = size / 2.0
    A = (cx - h, cy, cz - h)
    B = (cx + h, cy, cz - h)
    Cc = (cx + h, cy, cz + h)
    D = (cx - h, cy, cz + h)
    pts = np.array([A, B, Cc, D], dtype=np.float32)
    idx = np.array([0, 2, 1, 0, 3, 2] if facing_down else [0, 1, 2, 0, 2, 3], dtype=np.uint32)
    return Shape.triangle_mesh(Transform(), None, False, idx, pts)


POINT_LIGHT_POS = (0.0, 6.0, -2.0)


def c1_scene(seed: int | None = None, res: int = 512, spp_side: int = 2, n_spheres: int = 64):
    """Plain render: perspective camera at (0, 1.5, -6) looking at the
    origin, fov 60; ground quad (2 triangles, y = 0, [-10, 10]^2); matte
    spheres with r ~ U[0.1, 0.4], centre ~ U([-3,3] x [r,2] x [-3,3]),
    Kd ~ U[0.2, 0.8]^3; a point light of intensity 50 at POINT_LIGHT_POS and
    a 1x1 quad area light at y = 4 facing down with L = 10.
    Returns (prims, lights, camera, sampler)."""
    rng = PCG32(config_seed(1) if seed is None else seed)
    prims = []
    ground_pts = np.array([(-10, 0, -10), (10, 0, -10), (10, 0, 10), (-10, 0, 10)], np.float32)
    ground = Shape.triangle_mesh(Transform(), None, False, np.array([0, 1, 2, 0, 2, 3], np.uint32), ground_pts)
    prims.append(Primitive.geometric(ground, MatteMaterial((0.5, 0.5, 0.5))))
    u = rng.uniform(7 * n_spheres).reshape(n_spheres, 7)
    for i in range(n_spheres):
        r = 0.1 + 0.3 * u[i, 0]
        c = (-3.0 + 6.0 * u[i, 1], r + (2.0 - r) * u[i, 2], -3.0 + 6.0 * u[i, 3])
        kd = tuple(0.2 + 0.6 * u[i, 4:7])
        o2w = Transform.translate(c)
        s = Shape.sphere(o2w, o2w.inverse(), False, r, -r, r, 360.0)
        prims.append(Primitive.geometric(s, MatteMaterial(kd)))
    lights = [PointLight(Transform.translate(POINT_LIGHT_POS), (50.0, 50.0, 50.0))]
    area = DiffuseAreaLight(Transform(), (10.0, 10.0, 10.0))
    prims.append(Primitive.geometric_area_light(quad_light_mesh((0.0, 4.0, 0.0), 1.0), MatteMaterial((0, 0, 0)),
                                                area))
    lights.append(area)
    cam2world = Transform.look_at((0.0, 1.5, -6.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0)).inverse()
    film = Film.image(res, res, Filter.mean(0.5, 0.5))
    camera = Camera.perspective(cam2world, (-1.0, 1.0, -1.0, 1.0), 0.0, 1.0, 0.0, 1e30, 60.0, film)
    sampler = StratifiedSampler.stratified(0, res, 0, res, spp_side, spp_side, True, 0.0, 1.0)
    return prims, lights, camera, sampler


def heightfield_points(n_side: int = 708, extent: float = 8.0, seed: int | None = None) -> tuple:
    rng = PCG32(config_seed(2) if seed is None else seed)
    ph = rng.uniform(12) * 2.0 * math.pi
    xs = np.linspace(-extent, extent, n_side)
    X, Z = np.meshgrid(xs, xs, indexing="xy")
    H = np.zeros_like(X)
    for k in range(1, 7):
        H += 0.5 ** k * np.sin(2.0 ** k * X + ph[k - 1]) * np.cos(2.0 ** k * Z + ph[5 + k])
    pts = np.stack([X, H, Z], axis=-1).reshape(-1, 3).astype(np.float32)
    i = np.arange(n_side - 1)
    I, J = np.meshgrid(i, i, indexing="xy")
    v00 = (J * n_side + I).reshape(-1)
    v10 = v00 + 1
    v01 = v00 + n_side
    v11 = v01 + 1
    idx = np.stack([v00, v01, v10, v10, v01, v11], axis=1).reshape(-1).astype(np.uint32)
    return pts, idx, rng


def heightfield(n_side: int = 708, seed: int | None = None, res: int = 1024, spp_side: int = 4,
                n_rays: int = 1 << 22):
    """Large mesh: 708x708-vertex heightfield over [-8, 8]^2 with
    h = sum_k 0.5^k sin(2^k x + phi_k) cos(2^k z + psi_k), lit by a 4x4 quad
    area light at y = 6 (L = 8); camera at (0, 7, -14) looking at the
    origin, fov 50.  Returns (prims, lights, camera, sampler, rays); the
    rays start uniformly in the mesh AABB inflated by 1 and point uniformly
    over the sphere."""
    pts, idx, rng = heightfield_points(n_side, 8.0, seed)
    mesh = Shape.triangle_mesh(Transform(), None, False, idx, pts)
    prims = [Primitive.geometric(mesh, MatteMaterial((0.55, 0.5, 0.45)))]
    area = DiffuseAreaLight(Transform(), (8.0, 8.0, 8.0))
    prims.append(Primitive.geometric_area_light(quad_light_mesh((0.0, 6.0, 0.0), 4.0), MatteMaterial((0, 0, 0)),
                                                area))
    lights = [area]
    cam2world = Transform.look_at((0.0, 7.0, -14.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0)).inverse()
    film = Film.image(res, res, Filter.mean(0.5, 0.5))
    camera = Camera.perspective(cam2world, (-1.0, 1.0, -1.0, 1.0), 0.0, 1.0, 0.0, 1e30, 50.0, film)
    sampler = StratifiedSampler.stratified(0, res, 0, res, spp_side, spp_side, True, 0.0, 1.0)
    lo = pts.min(axis=0).astype(np.float64) - 1.0
    hi = pts.max(axis=0).astype(np.float64) + 1.0
    rays = incoherent_rays(rng, n_rays, lo, hi) if n_rays else None
    return prims, lights, camera, sampler, rays


def multi_scene(index: int, seed: int | None = None, tri_range=(1000, 256000), res_choices=(128, 256, 512),
                spp_choices=(1, 4, 16), max_spheres: int = 32):
    """One scene of the batched multi-scene workload: a random-triangle soup
    (as in ray_soup) with a log-uniform triangle count in tri_range, scaled
    to an extent E ~ U[1, 4]; 0..max_spheres matte spheres (r ~ E * U[0.05,
    0.2], centre ~ U[-E, E]^3); matte Kd ~ U[0.2, 0.8]^3 throughout; a point
    light (intensity 50 E^2 at (0, 2E, -E)) and a 1E x 1E quad area light at
    y = 1.5E facing down (L = 10).  Camera at (0, 0.5E, -3.5E) looking at the
    origin, fov 60; resolution and spp drawn from the choices (spp as n x n
    jittered strata).  Returns (prims, lights, camera, sampler)."""
    rng = PCG32(config_seed(3, index) if seed is None else seed)
    u = rng.uniform(8)
    lo, hi = math.log(tri_range[0]), math.log(tri_range[1])
    n_tris = int(round(math.exp(lo + (hi - lo) * u[0])))
    E = 1.0 + 3.0 * u[1]
    n_sph = min(int(u[2] * (max_spheres + 1)), max_spheres)
    res = res_choices[min(int(u[3] * len(res_choices)), len(res_choices) - 1)]
    spp = spp_choices[min(int(u[4] * len(spp_choices)), len(spp_choices) - 1)]
    side = int(round(math.sqrt(spp)))
    kd = tuple(0.2 + 0.6 * u[5:8])
    pts, idx = random_triangle_soup(rng, n_tris, extent=E, offset=0.05 * E)
    mesh = Shape.triangle_mesh(Transform(), None, False, idx, pts)
    prims = [Primitive.geometric(mesh, MatteMaterial(kd))]
    s = rng.uniform(7 * n_sph).reshape(n_sph, 7) if n_sph else np.zeros((0, 7))
    for i in range(n_sph):
        r = E * (0.05 + 0.15 * s[i, 0])
        c = tuple(E * (2.0 * s[i, 1:4] - 1.0))
        o2w = Transform.translate(c)
        prims.append(Primitive.geometric(Shape.sphere(o2w, o2w.inverse(), False, r, -r, r, 360.0),
                                         MatteMaterial(tuple(0.2 + 0.6 * s[i, 4:7]))))
    lights = [PointLight(Transform.translate((0.0, 2.0 * E, -E)), (50.0 * E * E,) * 3)]
    area = DiffuseAreaLight(Transform(), (10.0, 10.0, 10.0))
    prims.append(Primitive.geometric_area_light(quad_light_mesh((0.0, 1.5 * E, 0.0), E), MatteMaterial((0, 0, 0)),
                                                area))
    lights.append(area)
    cam2world = Transform.look_at((0.0, 0.5 * E, -3.5 * E), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0)).inverse()
    film = Film.image(res, res, Filter.mean(0.5, 0.5))
    camera = Camera.perspective(cam2world, (-1.0, 1.0, -1.0, 1.0), 0.0, 1.0, 0.0, 1e30, 60.0, film)
    sampler = StratifiedSampler.stratified(0, res, 0, res, side, side, True, 0.0, 1.0)
    return prims, lights, camera, sampler


def orbit_camera(camera, radius: float, azimuth: float, height: float | None = None, target=(0.0, 0.0, 0.0)):
    """The camera moved to a point on a circle around `target` (radius,
    azimuth in radians, height above the target: radius / 4 by default),
    looking at the target; film, fov and screen window unchanged."""
    h = radius / 4.0 if height is None else height
    eye = (target[0] + radius * math.sin(azimuth), target[1] + h, target[2] - radius * math.cos(azimuth))
    cam2world = Transform.look_at(eye, tuple(target), (0.0, 1.0, 0.0)).inverse()
    return Camera.perspective(cam2world, camera.screen_window, camera.shutter_open, camera.shutter_close,
                              camera.lens_radius, camera.focal_distance, camera.fov, camera.film)


def serving_requests(n: int, n_scenes: int, seed: int | None = None, render_fraction: float = 0.5):
    """The request stream of the serving workload: each request is a render
    (scene uniform, camera orbiting the scene's centre at radius U[4, 8] with
    a uniform azimuth, resolution from {128, 256, 512} squared, 1 or 4 spp)
    or a ray batch of 2^14..2^18 rays with origins in the scene bounds and
    uniform directions.  Returns dicts describing them; arrival times come
    from poisson_arrivals."""
    rng = PCG32(config_seed(4) if seed is None else seed)
    u = rng.uniform(6 * n).reshape(n, 6)
    out = []
    for k in range(n):
        scene = min(int(u[k, 0] * n_scenes), n_scenes - 1)
        if u[k, 1] < render_fraction:
            out.append({"kind": "render", "scene": scene, "res": (128, 256, 512)[min(int(u[k, 2] * 3), 2)],
                        "spp": (1, 4)[min(int(u[k, 3] * 2), 1)], "radius": 4.0 + 4.0 * u[k, 4],
                        "azimuth": 2.0 * math.pi * u[k, 5]})
        else:
            out.append({"kind": "query", "scene": scene, "n": 1 << (14 + min(int(u[k, 2] * 5), 4)),
                        "seed": config_seed(4, 1000 + k)})
    return out


def poisson_arrivals(n: int, rate: float, seed: int = 0) -> np.ndarray:
    """Arrival times (seconds from 0) of a Poisson process of `rate` per
    second: cumulative sums of exponential gaps drawn by inversion."""
    u = PCG32(seed).uniform(n)
    return np.cumsum(-np.log1p(-u) / rate)


def instanced_forest(n_instances: int = 64, tris_per_tree: int = 2000, seed: int | None = None, res: int = 128,
                     spp_side: int = 2):
    """Two definitions in instance space: a "tree" (a triangle soup cone of
    `tris_per_tree` triangles in y [0, 2], a sphere crown of radius 0.6 at
    y = 2.2, a disk base of radius 0.5 rotated to face +y) and a "post" (a
    cylinder of radius 0.15 along y with a 2-triangle cap).  Instance k:
    rotate(360 u0, y) and uniform scale 0.5 + u1, translated to
    (-8 + 16 u2, 0, -8 + 16 u3); even k use the tree.  Ground quad
    (y = 0, [-10, 10]^2), point light, quad area light at y = 6.  Returns
    (prims, lights, camera, sampler, flat) where `flat` has every instance
    copied out shape by shape with the composed transform (the same scene
    without instancing)."""
    rng = PCG32(config_seed(7) if seed is None else seed)
    n = tris_per_tree
    u = rng.uniform(12 * n).reshape(n, 12)
    h = 2.0 * u[:, 0]
    ang = 2.0 * math.pi * u[:, 1]
    rad = 0.6 * (1.0 - h / 2.0) * np.sqrt(u[:, 2])
    cen = np.stack([rad * np.cos(ang), h, rad * np.sin(ang)], axis=-1)
    off = (u[:, 3:12].reshape(n, 3, 3) * 2.0 - 1.0) * 0.08
    pts = (cen[:, None, :] + off).reshape(-1, 3).astype(np.float32)
    bark, leaf, stone = MatteMaterial((0.45, 0.3, 0.15)), MatteMaterial((0.2, 0.6, 0.25)), MatteMaterial((0.6,) * 3)
    tree = InstanceDefinition([
        Primitive.geometric(Shape.triangle_mesh(Transform(), None, False, np.arange(3 * n, dtype=np.uint32), pts),
                            leaf),
        Primitive.geometric(Shape.sphere(Transform.translate((0.0, 2.2, 0.0)), None, False, 0.6, -0.6, 0.6, 360.0),
                            leaf),
        Primitive.geometric(Shape.disk(Transform.rotate(-90.0, (1.0, 0.0, 0.0)), None, False, 0.01, 0.5, 0.0,
                                       360.0), bark),
    ])
    cap = np.array([(-0.2, 1.5, -0.2), (0.2, 1.5, -0.2), (0.2, 1.5, 0.2), (-0.2, 1.5, 0.2)], np.float32)
    post = InstanceDefinition([
        Primitive.geometric(Shape.cylinder(Transform.rotate(-90.0, (1.0, 0.0, 0.0)), None, False, 0.15, 0.0, 1.5,
                                           360.0), stone),
        Primitive.geometric(Shape.triangle_mesh(Transform(), None, False, np.array([0, 2, 1, 0, 3, 2], np.uint32),
                                                cap), stone),
    ])
    ground_pts = np.array([(-10, 0, -10), (10, 0, -10), (10, 0, 10), (-10, 0, 10)], np.float32)
    ground = Primitive.geometric(
        Shape.triangle_mesh(Transform(), None, False, np.array([0, 1, 2, 0, 2, 3], np.uint32), ground_pts),
        MatteMaterial((0.5, 0.5, 0.5)))
    prims, flat = [ground], [ground]
    v = rng.uniform(4 * n_instances).reshape(n_instances, 4)
    for k in range(n_instances):
        sc = 0.5 + float(v[k, 1])
        i2w = (Transform.translate((-8.0 + 16.0 * float(v[k, 2]), 0.0, -8.0 + 16.0 * float(v[k, 3])))
               * Transform.rotate(360.0 * float(v[k, 0]), (0.0, 1.0, 0.0)) * Transform.scale(sc, sc, sc))
        defn = tree if k % 2 == 0 else post
        prims.append(Primitive.transformed(defn, i2w.inverse()))
        for q in defn.prims:
            flat.append(Primitive.geometric(dataclasses.replace(q.shape, object_to_world=i2w * q.shape.object_to_world),
                                            q.material))
    lights = [PointLight(Transform.translate((3.0, 7.0, -4.0)), (120.0, 120.0, 120.0))]
    area = DiffuseAreaLight(Transform(), (8.0, 8.0, 8.0))
    lamp = Primitive.geometric_area_light(quad_light_mesh((0.0, 6.0, 0.0), 2.0), MatteMaterial((0, 0, 0)), area)
    prims.append(lamp)
    flat.append(lamp)
    lights.append(area)
    cam2world = Transform.look_at((0.0, 6.0, -14.0), (0.0, 0.5, 0.0), (0.0, 1.0, 0.0)).inverse()
    film = Film.image(res, res, Filter.mean(0.5, 0.5))
    camera = Camera.perspective(cam2world, (-1.0, 1.0, -1.0, 1.0), 0.0, 1.0, 0.0, 1e30, 55.0, film)
    sampler = StratifiedSampler.stratified(0, res, 0, res, spp_side, spp_side, True, 0.0, 1.0)
    return prims, lights, camera, sampler, flat
