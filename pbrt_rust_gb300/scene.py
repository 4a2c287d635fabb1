"""Host-side mirror of the reference's scene surface for the GPU path.

Names and argument meaning follow the crate: ``Shape::triangle_mesh`` /
``Shape::sphere`` (src/shape/mod.rs:170-190), ``Primitive::geometric``
(src/primitive/mod.rs:87-99), ``Aggregate::bvh`` / ``BVHAccelerator::new``
(src/primitive/aggregates/mod.rs:27-29, bvh.rs:334-363), ``PointLight``
(src/light/point.rs:16-35), ``MatteMaterial`` (src/material/matte.rs),
``Camera::perspective`` (src/camera/mod.rs:105-135), ``Film::image``
(src/camera/film.rs:77-122), ``Filter::mean`` (src/filter.rs:45-50) and
``Sampler::stratified`` (src/sampler/mod.rs:29-35).  The objects only
describe the scene; the work happens in the compiled library.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .transform import Transform


# ------------------------------------------------------------------ shapes --
@dataclass
class Shape:
    kind: int
    object_to_world: Transform
    reverse_orientation: bool = False
    points: np.ndarray | None = None   # (n, 3) float32, object space
    indices: np.ndarray | None = None  # (3m,) uint32
    radius: float = 1.0
    z0: float = -1.0
    z1: float = 1.0
    phi_max: float = 360.0
    height: float = 0.0        # disk
    inner_radius: float = 0.0  # disk
    definition: "InstanceDefinition | None" = None  # instance: the shared primitives

    @staticmethod
    def triangle_mesh(o2w: Transform, w2o: Transform | None, ro: bool, vi, p) -> "Shape":
        """Shape::triangle_mesh (src/shape/mod.rs:185-190); w2o is implied
        by o2w (its inverse)."""
        pts = np.ascontiguousarray(np.asarray(p, dtype=np.float32).reshape(-1, 3))
        idx = np.ascontiguousarray(np.asarray(vi, dtype=np.uint32).reshape(-1))
        if idx.size % 3:
            raise ValueError("vertex index count must be a multiple of 3 (mesh.rs:303)")
        if idx.size and int(idx.max()) >= len(pts):
            raise ValueError("vertex index out of range")
        return Shape(abi.SHAPE_TRIANGLE_MESH, o2w, bool(ro), points=pts, indices=idx)

    @staticmethod
    def sphere(o2w: Transform, w2o: Transform | None, ro: bool, rad: float, z0: float, z1: float,
               pm: float) -> "Shape":
        """Shape::sphere (src/shape/mod.rs:170-173)."""
        if not rad > 0:
            raise ValueError("sphere radius must be positive (sphere.rs:30)")
        return Shape(abi.SHAPE_SPHERE, o2w, bool(ro), radius=float(rad), z0=float(z0), z1=float(z1),
                     phi_max=float(pm))

    @staticmethod
    def disk(o2w: Transform, w2o: Transform | None, ro: bool, height: float, radius: float, inner_radius: float,
             phi_max: float) -> "Shape":
        """Disk::new (src/shape/disk.rs:24-34)."""
        return Shape(abi.SHAPE_DISK, o2w, bool(ro), radius=float(radius), phi_max=float(phi_max),
                     height=float(height), inner_radius=float(inner_radius))

    @staticmethod
    def cylinder(o2w: Transform, w2o: Transform | None, ro: bool, radius: float, z0: float, z1: float,
                 phi_max: float) -> "Shape":
        """Cylinder::new (src/shape/cylinder.rs:26-36)."""
        return Shape(abi.SHAPE_CYLINDER, o2w, bool(ro), radius=float(radius), z0=float(z0), z1=float(z1),
                     phi_max=float(phi_max))

    def num_primitives(self) -> int:
        return len(self.indices) // 3 if self.kind == abi.SHAPE_TRIANGLE_MESH else 1

    def num_ids(self) -> int:
        """Hit ids the shape takes: an instance takes one per refined
        primitive of its definition."""
        if self.kind == abi.SHAPE_INSTANCE:
            return self.definition.num_primitives()
        return self.num_primitives()


@dataclass(eq=False)
class InstanceDefinition:
    """The primitives of one ObjectBegin ... ObjectEnd block
    (src/main.rs:714-733) in instance space, shared by all its instances:
    one BVH over them is built once per scene.  They hold no area lights
    and no instances."""
    prims: list

    def num_primitives(self) -> int:
        return sum(p.shape.num_primitives() for p in self.prims)


@dataclass
class MatteMaterial:
    """MatteMaterial with constant textures (src/material/matte.rs:30-51)."""
    kd: tuple = (0.5, 0.5, 0.5)
    sigma: float = 0.0


@dataclass
class PointLight:
    """PointLight::new(l2w, intensity) (src/light/point.rs:78-83)."""
    light_to_world: Transform
    intensity: tuple


@dataclass
class DiffuseAreaLight:
    """Diffuse area light over one triangle mesh (pbrt-v2 semantics; the
    reference's AreaLight is a stub, src/area_light.rs:8-24)."""
    light_to_world: Transform
    radiance: tuple
    shape: Shape | None = None


@dataclass
class Primitive:
    shape: Shape
    material: MatteMaterial = field(default_factory=MatteMaterial)
    area_light: DiffuseAreaLight | None = None

    @staticmethod
    def geometric(s: Shape, mtl: MatteMaterial | None = None) -> "Primitive":
        return Primitive(s, mtl or MatteMaterial())

    @staticmethod
    def simple(s: Shape) -> "Primitive":
        return Primitive(s, MatteMaterial())

    @staticmethod
    def transformed(defn: InstanceDefinition, world_to_primitive: Transform) -> "Primitive":
        """Primitive::transformed (src/primitive/mod.rs:101-106) with a
        static transform: TransformedPrimitive (transformed.rs:14-59) over
        the definition's aggregate.  Hits inside it report the id
        (first id of the instance) + (refined index inside the
        definition)."""
        if not isinstance(defn, InstanceDefinition):
            raise TypeError("an instance refers to an InstanceDefinition")
        if not defn.prims:
            raise ValueError("instance of an empty definition")
        for p in defn.prims:
            if p.area_light is not None or p.shape.kind == abi.SHAPE_INSTANCE:
                raise ValueError("instance definitions hold neither area lights nor instances")
        shape = Shape(abi.SHAPE_INSTANCE, world_to_primitive.inverse(), definition=defn)
        return Primitive(shape, MatteMaterial())

    @staticmethod
    def geometric_area_light(s: Shape, mtl: MatteMaterial, al: DiffuseAreaLight) -> "Primitive":
        if s.kind != abi.SHAPE_TRIANGLE_MESH:
            raise ValueError("area lights are supported on triangle meshes")
        al.shape = s
        return Primitive(s, mtl, al)


class SceneDescription:
    """Marshals primitives, materials and lights into a PbrtSceneDesc; keeps
    every array it points to alive for the lifetime of the object."""

    def __init__(self, prims: list[Primitive], lights: list = (), max_prims: int = 4, split_method: str = "sah",
                 aggregate_only: bool = False):
        self.prims = list(prims)
        self.lights = list(lights)
        self._keep = []
        mats: list[MatteMaterial] = []
        mat_index: dict[int, int] = {}
        defs: list[InstanceDefinition] = []
        def_index: dict[int, int] = {}
        for p in self.prims:
            d = p.shape.definition if p.shape.kind == abi.SHAPE_INSTANCE else None
            if d is not None and id(d) not in def_index:
                def_index[id(d)] = len(defs)
                defs.append(d)
        for p in self.prims + [q for d in defs for q in d.prims]:
            if p.shape.kind != abi.SHAPE_INSTANCE and id(p.material) not in mat_index:
                mat_index[id(p.material)] = len(mats)
                mats.append(p.material)
        light_index = {id(l): i for i, l in enumerate(self.lights)}
        shape_index = {id(p.shape): i for i, p in enumerate(self.prims)}
        n = len(self.prims)
        self.shapes = self._shape_array(self.prims, mat_index, def_index, light_index, aggregate_only)
        # instance definitions, their shapes marshalled like the scene's
        self.definitions = defs
        self.def_shapes = [self._shape_array(d.prims, mat_index, {}, {}, True) for d in defs]
        self.instance_descs = (abi.PbrtInstanceDesc * max(len(defs), 1))()
        for k, d in enumerate(defs):
            self.instance_descs[k].shapes = self.def_shapes[k]
            self.instance_descs[k].n_shapes = len(d.prims)
        self.materials = (abi.PbrtMaterialDesc * max(len(mats), 1))()
        for i, m in enumerate(mats):
            self.materials[i].kd[:] = [float(c) for c in m.kd]
            self.materials[i].sigma = float(m.sigma)
        self.light_descs = (abi.PbrtLightDesc * max(len(self.lights), 1))()
        for i, l in enumerate(self.lights):
            d = self.light_descs[i]
            d.light_to_world = l.light_to_world.to_abi()
            if isinstance(l, PointLight):
                d.kind = abi.LIGHT_POINT
                d.spectrum[:] = [float(c) for c in l.intensity]
                d.shape = -1
            elif isinstance(l, DiffuseAreaLight):
                d.kind = abi.LIGHT_DIFFUSE_AREA
                d.spectrum[:] = [float(c) for c in l.radiance]
                if l.shape is None or id(l.shape) not in shape_index:
                    raise ValueError("area light has no emitting primitive in the scene")
                d.shape = shape_index[id(l.shape)]
            else:
                raise TypeError(f"unsupported light {type(l).__name__}")
        if split_method not in abi.SPLIT_METHODS:
            print(f'Warning: BVH split method {split_method} unknown. Using "SAH"')
        self.split_method = split_method
        self.desc = abi.PbrtSceneDesc()
        self.desc.shapes = self.shapes
        self.desc.n_shapes = n
        self.desc.materials = self.materials
        self.desc.n_materials = len(mats)
        self.desc.lights = self.light_descs
        self.desc.n_lights = len(self.lights)
        self.desc.max_prims_in_node = int(max_prims)
        self.desc.split_method = abi.SPLIT_METHODS.get(split_method, 0)
        self.desc.instances = self.instance_descs
        self.desc.n_instances = len(defs)

    def _shape_array(self, prims, mat_index, def_index, light_index, aggregate_only):
        arr = (abi.PbrtShapeDesc * max(len(prims), 1))()
        for i, p in enumerate(prims):
            s = p.shape
            d = arr[i]
            d.kind = s.kind
            d.reverse_orientation = int(s.reverse_orientation)
            d.object_to_world = s.object_to_world.to_abi()
            if s.kind == abi.SHAPE_TRIANGLE_MESH:
                self._keep += [s.points, s.indices]
                d.points = abi.f32p(s.points)
                d.n_points = len(s.points)
                d.indices = abi.u32p(s.indices)
                d.n_indices = len(s.indices)
            d.radius, d.z0, d.z1, d.phi_max_deg = s.radius, s.z0, s.z1, s.phi_max
            d.height, d.inner_radius = s.height, s.inner_radius
            if s.kind == abi.SHAPE_INSTANCE:
                if id(s.definition) not in def_index:
                    raise ValueError("instance definitions hold no instances")
                d.instance = def_index[id(s.definition)]
                d.material = 0
            else:
                d.instance = -1
                d.material = mat_index[id(p.material)]
            if p.area_light is not None and not aggregate_only:
                if id(p.area_light) not in light_index:
                    raise ValueError("an area light of a primitive is missing from the scene's lights")
                d.area_light = light_index[id(p.area_light)]
            else:
                d.area_light = -1
        return arr

    def num_primitives(self) -> int:
        return sum(p.shape.num_primitives() for p in self.prims)

    def num_ids(self) -> int:
        """Ids hits report: refined primitives with every instance counted
        out (equal to num_primitives without instances)."""
        return sum(p.shape.num_ids() for p in self.prims)


# ---------------------------------------------------------- camera & film --
@dataclass
class Filter:
    """The film's reconstruction filter (src/filter.rs:44-85): ``kind`` is a
    key of abi.FILTERS; p0 = alpha (gaussian), B (mitchell) or tau
    (lanczos), p1 = C (mitchell)."""
    x_width: float = 0.5
    y_width: float = 0.5
    kind: str = "box"
    p0: float = 0.0
    p1: float = 0.0

    @staticmethod
    def mean(xw: float, yw: float) -> "Filter":
        return Filter(float(xw), float(yw))

    @staticmethod
    def triangle(xw: float, yw: float) -> "Filter":
        return Filter(float(xw), float(yw), "triangle")

    @staticmethod
    def gaussian(xw: float, yw: float, a: float) -> "Filter":
        return Filter(float(xw), float(yw), "gaussian", float(a))

    @staticmethod
    def mitchell(xw: float, yw: float, b: float, c: float) -> "Filter":
        return Filter(float(xw), float(yw), "mitchell", float(b), float(c))

    @staticmethod
    def lanczos(xw: float, yw: float, tau: float) -> "Filter":
        return Filter(float(xw), float(yw), "lanczos", float(tau))


@dataclass
class Film:
    """Film::image (src/camera/film.rs:77-122)."""
    x_res: int
    y_res: int
    filter: Filter = field(default_factory=Filter)
    crop: tuple = (0.0, 1.0, 0.0, 1.0)
    filename: str = ""

    @staticmethod
    def image(xres: int, yres: int, filt: Filter, crop=(0.0, 1.0, 0.0, 1.0), filename: str = "",
              open_window: bool = False) -> "Film":
        if open_window:
            raise NotImplementedError("display windows are not supported (film.rs:99-102 is a stub too)")
        return Film(int(xres), int(yres), filt, tuple(float(c) for c in crop), filename)

    def pixel_extent(self) -> tuple[int, int, int, int]:
        """film.rs:81-84, 301-309 with f32 arithmetic."""
        f32 = np.float32
        xs = int(math.ceil(f32(self.x_res) * f32(self.crop[0])))
        xc = max(int(math.ceil(f32(self.x_res) * f32(self.crop[1]))) - xs, 1)
        ys = int(math.ceil(f32(self.y_res) * f32(self.crop[2])))
        yc = max(int(math.ceil(f32(self.y_res) * f32(self.crop[3]))) - ys, 1)
        return xs, xs + xc, ys, ys + yc


@dataclass
class Camera:
    """Camera::perspective (src/camera/mod.rs:105-135) with a static
    camera-to-world transform."""
    camera_to_world: Transform
    screen_window: tuple
    shutter_open: float
    shutter_close: float
    lens_radius: float
    focal_distance: float
    fov: float
    film: Film

    @staticmethod
    def perspective(cam2world: Transform, screen_window, sopen: float, sclose: float, lensr: float,
                    focald: float, fov: float, film: Film) -> "Camera":
        return Camera(cam2world, tuple(float(c) for c in screen_window), float(sopen), float(sclose),
                      float(lensr), float(focald), float(fov), film)

    def to_abi(self) -> abi.PbrtCameraDesc:
        d = abi.PbrtCameraDesc()
        d.camera_to_world = self.camera_to_world.to_abi()
        d.fov_deg = self.fov
        d.screen_window[:] = list(self.screen_window)
        d.lens_radius = self.lens_radius
        d.focal_distance = self.focal_distance
        d.shutter_open = self.shutter_open
        d.shutter_close = self.shutter_close
        d.x_res = self.film.x_res
        d.y_res = self.film.y_res
        d.crop_window[:] = list(self.film.crop)
        d.filter_x_width = self.film.filter.x_width
        d.filter_y_width = self.film.filter.y_width
        d.filter_kind = abi.FILTERS[self.film.filter.kind]
        d.filter_p0 = self.film.filter.p0
        d.filter_p1 = self.film.filter.p1
        return d


def default_screen_window(xres: int, yres: int) -> tuple:
    """pbrt-v2's default: the shorter image axis spans [-1, 1]."""
    frame = xres / yres
    if frame > 1.0:
        return (-frame, frame, -1.0, 1.0)
    return (-1.0, 1.0, -1.0 / frame, 1.0 / frame)


@dataclass
class StratifiedSampler:
    """Sampler::stratified (src/sampler/mod.rs:29-35)."""
    x_start: int
    x_end: int
    y_start: int
    y_end: int
    x_samples: int
    y_samples: int
    jitter: bool = True
    shutter_open: float = 0.0
    shutter_close: float = 1.0

    @staticmethod
    def stratified(x_start, x_end, y_start, y_end, xs, ys, jitter, sopen, sclose) -> "StratifiedSampler":
        return StratifiedSampler(int(x_start), int(x_end), int(y_start), int(y_end), int(xs), int(ys),
                                 bool(jitter), float(sopen), float(sclose))

    def samples_per_pixel(self) -> int:
        return self.x_samples * self.y_samples

    def to_abi(self, num_tasks: int) -> abi.PbrtSamplerDesc:
        d = abi.PbrtSamplerDesc()
        d.x_start, d.x_end, d.y_start, d.y_end = self.x_start, self.x_end, self.y_start, self.y_end
        d.x_samples, d.y_samples = self.x_samples, self.y_samples
        d.jitter = int(self.jitter)
        d.shutter_open, d.shutter_close = self.shutter_open, self.shutter_close
        d.num_tasks = int(num_tasks)
        return d


def default_num_tasks(x_res: int, y_res: int, num_cpus: int = 8) -> int:
    """SamplerRenderer::new's task count (src/sampler_renderer.rs:39-44),
    ceil(log2(max(32 * num_cpus, npix / 256))), for a fixed core count so
    random streams do not depend on the host."""
    x = max(32 * num_cpus, (x_res * y_res) // 256)
    return (x - 1).bit_length() if x > 1 else 0
