"""Scene ingestion: ParamSet, the pbrt scene-description API and a parser
for pbrt-v2 scene files.

The reference crate declares this front end but leaves it stubbed: the
parser returns nothing (src/main.rs:802), ``make_accelerator`` and
``make_area_light`` are unimplemented (main.rs:311-314, 331-333) and only
the "sphere" shape exists (main.rs:316-329).  This module follows the
reference's API surface (``Pbrt`` state machine, main.rs:380-800;
``ParamSet``, src/params.rs; the factories of main.rs:288-329) and fills the
stubs with pbrt-v2 semantics, producing the same ``Primitive`` / light /
``Camera`` / ``StratifiedSampler`` objects the programmatic interface
builds, which then render through ``GpuSamplerRenderer`` (or the oracle).

Supported: Identity, Translate, Rotate, Scale, LookAt, ConcatTransform,
Transform, CoordinateSystem, CoordSysTransform, ActiveTransform,
TransformTimes (static transforms only), Camera "perspective", Film
"image", PixelFilter box/triangle/gaussian/mitchell/sinc, Sampler
"stratified", SurfaceIntegrator "directlighting"/"whitted" (both the
direct-lighting Li), Accelerator "bvh" (maxnodeprims, splitmethod),
WorldBegin/WorldEnd, AttributeBegin/End, TransformBegin/End,
ReverseOrientation, Material / MakeNamedMaterial / NamedMaterial "matte",
Texture "constant", LightSource "point", AreaLightSource "diffuse" on
triangle meshes, Shape "sphere", "disk", "cylinder" and "trianglemesh", ObjectBegin/End and
ObjectInstance (TransformedPrimitive instances sharing one BVH per
definition, see ``object_instance``), Include.
Anything else raises ``NotImplementedError`` (the reference panics).
"""
from __future__ import annotations

import dataclasses
import os
import re
from dataclasses import dataclass, field

import numpy as np

from .scene import (Camera, DiffuseAreaLight, Film, Filter, InstanceDefinition, MatteMaterial, PointLight,
                    Primitive, Shape, StratifiedSampler, default_num_tasks)
from .transform import Transform


# ------------------------------------------------------------------ ParamSet
class ParamSet:
    """src/params.rs: typed, named parameter lists."""

    TYPES = ("bool", "integer", "float", "point", "vector", "normal", "rgb", "color", "xyz", "blackbody",
             "spectrum", "string", "texture")

    def __init__(self):
        self._p: dict[str, tuple[str, list]] = {}

    def add(self, ty: str, name: str, values) -> None:
        if ty == "color":
            ty = "rgb"
        if ty == "point3":
            ty = "point"
        if ty not in self.TYPES:
            raise ValueError(f"unknown parameter type {ty!r}")
        if name in self._p:
            print(f"WARNING: Param {name} already exists!")  # params.rs:31-35
        self._p[name] = (ty, list(values))

    def _find(self, ty: str, name: str):
        v = self._p.get(name)
        return v[1] if v is not None and v[0] == ty else None

    def find_one_float(self, name: str, default: float) -> float:
        v = self._find("float", name)
        return float(v[0]) if v else default

    def find_one_int(self, name: str, default: int) -> int:
        v = self._find("integer", name)
        return int(v[0]) if v else default

    def find_one_bool(self, name: str, default: bool) -> bool:
        v = self._find("bool", name)
        return bool(v[0]) if v else default

    def find_one_string(self, name: str, default: str) -> str:
        v = self._find("string", name)
        return str(v[0]) if v else default

    def find_one_point(self, name: str, default) -> tuple:
        v = self._find("point", name)
        return tuple(float(x) for x in v[:3]) if v and len(v) >= 3 else tuple(default)

    def find_float(self, name: str):
        return self._find("float", name)

    def find_int(self, name: str):
        return self._find("integer", name)

    def find_point(self, name: str):
        return self._find("point", name)

    def find_one_texture(self, name: str, default: str = "") -> str:
        v = self._find("texture", name)
        return str(v[0]) if v else default

    def find_one_spectrum(self, name: str, default) -> tuple:
        """RGB spectra (params.rs:223-251); XYZ and blackbody are not
        supported by the RGB renderer."""
        v = self._p.get(name)
        if v is None:
            return tuple(default)
        ty, vals = v
        if ty == "rgb" and len(vals) >= 3:
            return tuple(float(x) for x in vals[:3])
        if ty == "float" and vals:  # Spectrum::from(f32) of a single value
            return (float(vals[0]),) * 3
        raise NotImplementedError(f"spectrum parameter {name!r} of type {ty}")

    def names(self) -> list[str]:
        return list(self._p)


class TextureParams:
    """params.rs:271-360: the shape's parameters first, then the
    material's; spectrum and float textures are constant ones."""

    def __init__(self, geom: ParamSet, mat: ParamSet, float_tex: dict, spec_tex: dict):
        self.geom, self.mat, self.float_tex, self.spec_tex = geom, mat, float_tex, spec_tex

    def spectrum(self, name: str, default) -> tuple:
        for ps in (self.geom, self.mat):
            tex = ps.find_one_texture(name)
            if tex:
                if tex not in self.spec_tex:
                    raise KeyError(f"unknown spectrum texture {tex!r}")
                return self.spec_tex[tex]
            if name in ps.names():
                return ps.find_one_spectrum(name, default)
        return tuple(default)

    def float(self, name: str, default: float) -> float:
        for ps in (self.geom, self.mat):
            tex = ps.find_one_texture(name)
            if tex:
                if tex not in self.float_tex:
                    raise KeyError(f"unknown float texture {tex!r}")
                return self.float_tex[tex]
            if name in ps.names():
                return ps.find_one_float(name, default)
        return default


# ------------------------------------------------------------------ factories
def make_material(name: str, tp: TextureParams) -> MatteMaterial:
    """main.rs:288-296."""
    if name == "matte":
        return MatteMaterial(tp.spectrum("Kd", (0.5, 0.5, 0.5)), tp.float("sigma", 0.0))
    raise NotImplementedError(f"Unknown material type: {name}")


def make_light(name: str, light_to_world: Transform, ps: ParamSet) -> PointLight:
    """main.rs:298-309: the point light sits at `from`, moved by the light's
    transform: Transform::translate(from) * light_to_world."""
    if name == "point":
        i = ps.find_one_spectrum("I", (1.0, 1.0, 1.0))
        sc = ps.find_one_spectrum("scale", (1.0, 1.0, 1.0))
        p = ps.find_one_point("from", (0.0, 0.0, 0.0))
        l2w = Transform.translate(p) * light_to_world
        f32 = np.float32
        return PointLight(l2w, tuple(float(f32(a) * f32(b)) for a, b in zip(i, sc)))
    raise NotImplementedError(f"Unknown light type: {name}")


def make_shape(name: str, o2w: Transform, w2o: Transform, ro: bool, ps: ParamSet) -> Shape:
    """main.rs:316-329, plus "trianglemesh" (pbrt-v2's `indices` / `P`;
    normals and uvs are not used by the reference's Triangle, which takes
    the default uvs, mesh.rs:74-87)."""
    if name == "sphere":
        radius = ps.find_one_float("radius", 1.0)
        zmin = ps.find_one_float("zmin", -radius)
        zmax = ps.find_one_float("zmax", radius)
        phimax = ps.find_one_float("phimax", 360.0)
        return Shape.sphere(o2w, w2o, ro, radius, zmin, zmax, phimax)
    if name == "disk":  # pbrt-v2 defaults
        return Shape.disk(o2w, w2o, ro, ps.find_one_float("height", 0.0), ps.find_one_float("radius", 1.0),
                          ps.find_one_float("innerradius", 0.0), ps.find_one_float("phimax", 360.0))
    if name == "cylinder":
        return Shape.cylinder(o2w, w2o, ro, ps.find_one_float("radius", 1.0), ps.find_one_float("zmin", -1.0),
                              ps.find_one_float("zmax", 1.0), ps.find_one_float("phimax", 360.0))
    if name == "trianglemesh":
        vi = ps.find_int("indices")
        p = ps.find_point("P")
        if vi is None or p is None:
            raise ValueError('trianglemesh needs "integer indices" and "point P"')
        if len(p) % 3:
            raise ValueError('"point P" needs a multiple of 3 values')
        return Shape.triangle_mesh(o2w, w2o, ro, np.asarray(vi, np.uint32), np.asarray(p, np.float32).reshape(-1, 3))
    raise NotImplementedError(f"Unknown shape type: {name}")


def make_filter(name: str, ps: ParamSet) -> Filter:
    """pbrt-v2's filter factories over src/filter.rs:44-85."""
    if name == "box":
        return Filter.mean(ps.find_one_float("xwidth", 0.5), ps.find_one_float("ywidth", 0.5))
    if name == "triangle":
        return Filter.triangle(ps.find_one_float("xwidth", 2.0), ps.find_one_float("ywidth", 2.0))
    if name == "gaussian":
        return Filter.gaussian(ps.find_one_float("xwidth", 2.0), ps.find_one_float("ywidth", 2.0),
                               ps.find_one_float("alpha", 2.0))
    if name == "mitchell":
        return Filter.mitchell(ps.find_one_float("xwidth", 2.0), ps.find_one_float("ywidth", 2.0),
                               ps.find_one_float("B", 1.0 / 3.0), ps.find_one_float("C", 1.0 / 3.0))
    if name == "sinc":
        return Filter.lanczos(ps.find_one_float("xwidth", 4.0), ps.find_one_float("ywidth", 4.0),
                              ps.find_one_float("tau", 3.0))
    raise NotImplementedError(f"Unknown filter type: {name}")


# ------------------------------------------------------------------ API state
STATE_UNINITIALIZED, STATE_OPTIONS_BLOCK, STATE_WORLD_BLOCK = 0, 1, 2


@dataclass
class GraphicsState:
    """main.rs:236-263."""
    material: str = "matte"
    material_params: ParamSet = field(default_factory=ParamSet)
    float_textures: dict = field(default_factory=dict)
    spectrum_textures: dict = field(default_factory=dict)
    named_materials: dict = field(default_factory=dict)
    current_named_material: str | None = None
    area_light: str = ""
    area_light_params: ParamSet = field(default_factory=ParamSet)
    reverse_orientation: bool = False

    def copy(self) -> "GraphicsState":
        return GraphicsState(self.material, self.material_params, dict(self.float_textures),
                             dict(self.spectrum_textures), dict(self.named_materials), self.current_named_material,
                             self.area_light, self.area_light_params, self.reverse_orientation)

    def create_material(self, params: ParamSet) -> MatteMaterial:
        """main.rs:265-277."""
        if self.current_named_material in self.named_materials:
            return self.named_materials[self.current_named_material]
        tp = TextureParams(params, self.material_params, self.float_textures, self.spectrum_textures)
        return make_material(self.material, tp)


@dataclass
class Frame:
    """What WorldEnd hands to the renderer (main.rs:774-800): the scene's
    primitives and lights, camera, sampler and accelerator settings."""
    primitives: list
    lights: list
    camera: Camera
    sampler: StratifiedSampler
    max_prims: int = 4
    split_method: str = "sah"
    num_tasks: int = 0

    def render(self, out=None, stream=None):
        """Renderer::render on the device (GpuSamplerRenderer); writes the
        film's file when it names one."""
        from .gpu import GpuSamplerRenderer, GpuScene
        scene = GpuScene(self.primitives, self.lights, self.max_prims, self.split_method)
        return GpuSamplerRenderer(self.sampler, self.camera, num_tasks=self.num_tasks).render(scene, out=out,
                                                                                              stream=stream)


class Pbrt:
    """The scene-description API (main.rs:335-800).  Every WorldEnd appends
    a Frame to ``frames`` (and renders it when ``render_on_world_end``)."""

    MAX_TRANSFORMS = 2

    def __init__(self, render_on_world_end: bool = False):
        self.render_on_world_end = render_on_world_end
        self.frames: list[Frame] = []
        self.state = STATE_OPTIONS_BLOCK
        self.ctm = [Transform(), Transform()]
        self.active = [True, True]
        self.named_coordinate_systems: dict[str, list] = {}
        self.gs = GraphicsState()
        self.pushed_gs: list = []
        self.pushed_ctm: list = []
        self.pushed_active: list = []
        self._reset_options()

    def _reset_options(self):
        self.transform_start_time, self.transform_end_time = 0.0, 1.0
        self.filter = ("box", ParamSet())
        self.film = ("image", ParamSet())
        self.sampler = ("stratified", ParamSet())  # the device renders with the stratified sampler only
        self.accelerator = ("bvh", ParamSet())
        self.surface_integrator = ("directlighting", ParamSet())
        self.camera = ("perspective", ParamSet())
        self.camera_to_world = [Transform(), Transform()]
        self.lights: list = []
        self.primitives: list = []
        self.instances: dict[str, list] = {}
        self.definitions: dict[str, InstanceDefinition] = {}  # shared by the instances of a name
        self.current_instance: str | None = None

    def _verify(self, want: int, what: str):
        if self.state != want:
            where = "world" if want == STATE_WORLD_BLOCK else "options"
            raise RuntimeError(f"{what} is only allowed inside the {where} block")

    def _apply(self, f):
        for i in range(self.MAX_TRANSFORMS):
            if self.active[i]:
                self.ctm[i] = f(self.ctm[i])

    # transforms (main.rs:426-519)
    def identity(self):
        self._apply(lambda t: Transform())

    def translate(self, dx, dy, dz):
        self._apply(lambda t: t * Transform.translate((dx, dy, dz)))

    def rotate(self, angle, ax, ay, az):
        self._apply(lambda t: t * Transform.rotate(angle, (ax, ay, az)))

    def scale(self, sx, sy, sz):
        self._apply(lambda t: t * Transform.scale(sx, sy, sz))

    def look_at(self, ex, ey, ez, lx, ly, lz, ux, uy, uz):
        self._apply(lambda t: t * Transform.look_at((ex, ey, ez), (lx, ly, lz), (ux, uy, uz)))

    def concat_transform(self, xf):
        """main.rs:467-476: xf holds the matrix row by row."""
        self._apply(lambda t: t * Transform.from_matrix(np.asarray(xf, np.float32).reshape(4, 4)))

    def transform(self, xf):
        """main.rs:478-487."""
        self._apply(lambda t: Transform.from_matrix(np.asarray(xf, np.float32).reshape(4, 4)))

    def coordinate_system(self, name: str):
        self.named_coordinate_systems[name] = list(self.ctm)

    def coord_sys_transform(self, name: str):
        if name in self.named_coordinate_systems:
            self.ctm = list(self.named_coordinate_systems[name])
        else:
            print(f"WARNING: No coordinate system named {name}")

    def active_transform_all(self):
        self.active = [True, True]

    def active_transform_start_time(self):
        self.active = [True, False]

    def active_transform_end_time(self):
        self.active = [False, True]

    def transform_times(self, start, end):
        self._verify(STATE_OPTIONS_BLOCK, "TransformTimes")
        self.transform_start_time, self.transform_end_time = float(start), float(end)

    # options (main.rs:521-564)
    def pixel_filter(self, name, ps):
        self._verify(STATE_OPTIONS_BLOCK, "PixelFilter")
        self.filter = (name, ps)

    def film_(self, name, ps):
        self._verify(STATE_OPTIONS_BLOCK, "Film")
        self.film = (name, ps)

    def sampler_(self, name, ps):
        self._verify(STATE_OPTIONS_BLOCK, "Sampler")
        self.sampler = (name, ps)

    def accelerator_(self, name, ps):
        self._verify(STATE_OPTIONS_BLOCK, "Accelerator")
        self.accelerator = (name, ps)

    def surface_integrator_(self, name, ps):
        self._verify(STATE_OPTIONS_BLOCK, "SurfaceIntegrator")
        self.surface_integrator = (name, ps)

    def volume_integrator_(self, name, ps):
        self._verify(STATE_OPTIONS_BLOCK, "VolumeIntegrator")  # no media on the path (D2)

    def renderer_(self, name, ps):
        self._verify(STATE_OPTIONS_BLOCK, "Renderer")
        if name != "sampler":
            raise NotImplementedError(f"renderer {name!r}: only the sampler renderer exists")

    def camera_(self, name, ps):
        self._verify(STATE_OPTIONS_BLOCK, "Camera")
        self.camera = (name, ps)
        self.camera_to_world = [t.inverse() for t in self.ctm]
        self.named_coordinate_systems["camera"] = list(self.camera_to_world)

    def world_begin(self):
        """main.rs:765-772."""
        self._verify(STATE_OPTIONS_BLOCK, "WorldBegin")
        self.state = STATE_WORLD_BLOCK
        self.active_transform_all()
        self.ctm = [Transform(), Transform()]
        self.named_coordinate_systems["world"] = list(self.ctm)

    # attributes (main.rs:394-424)
    def attribute_begin(self):
        self._verify(STATE_WORLD_BLOCK, "AttributeBegin")
        self.pushed_gs.append(self.gs.copy())
        self.pushed_ctm.append(list(self.ctm))
        self.pushed_active.append(list(self.active))

    def attribute_end(self):
        self._verify(STATE_WORLD_BLOCK, "AttributeEnd")
        if not self.pushed_gs:
            print("WARNING: Unmatched pbrt_attribute_end encountered. Ignoring.")
            return
        self.gs = self.pushed_gs.pop()
        self.ctm = self.pushed_ctm.pop()
        self.active = self.pushed_active.pop()

    def transform_begin(self):
        self._verify(STATE_WORLD_BLOCK, "TransformBegin")
        self.pushed_ctm.append(list(self.ctm))

    def transform_end(self):
        self._verify(STATE_WORLD_BLOCK, "TransformEnd")
        if not self.pushed_ctm:
            print("WARNING: Unmatched pbrt_transform_end encountered. Ignoring.")
            return
        self.ctm = self.pushed_ctm.pop()

    def reverse_orientation(self):
        self._verify(STATE_WORLD_BLOCK, "ReverseOrientation")
        self.gs.reverse_orientation = not self.gs.reverse_orientation

    # materials and textures (main.rs:566-620)
    def texture(self, name, ty, texname, ps):
        self._verify(STATE_WORLD_BLOCK, "Texture")
        if texname != "constant":
            raise NotImplementedError(f"texture class {texname!r}: only constant textures exist")
        if ty == "float":
            self.gs.float_textures[name] = ps.find_one_float("value", 1.0)
        elif ty in ("spectrum", "color"):
            self.gs.spectrum_textures[name] = ps.find_one_spectrum("value", (1.0, 1.0, 1.0))
        else:
            raise ValueError(f"texture type {ty!r}")

    def material(self, name, ps):
        self._verify(STATE_WORLD_BLOCK, "Material")
        self.gs.material = name
        self.gs.material_params = ps
        self.gs.current_named_material = None

    def make_named_material(self, name, ps):
        self._verify(STATE_WORLD_BLOCK, "MakeNamedMaterial")
        kind = ps.find_one_string("type", "")
        if not kind:
            raise ValueError("No parameter string \"type\" found in MakeNamedMaterial")
        tp = TextureParams(ps, ParamSet(), self.gs.float_textures, self.gs.spectrum_textures)
        self.gs.named_materials[name] = make_material(kind, tp)

    def named_material(self, name):
        self._verify(STATE_WORLD_BLOCK, "NamedMaterial")
        self.gs.current_named_material = name

    # lights and shapes (main.rs:622-712)
    def light_source(self, name, ps):
        self._verify(STATE_WORLD_BLOCK, "LightSource")
        self.lights.append(make_light(name, self.ctm[0], ps))

    def area_light_source(self, name, ps):
        self._verify(STATE_WORLD_BLOCK, "AreaLightSource")
        self.gs.area_light = name
        self.gs.area_light_params = ps

    def shape(self, name, ps):
        """main.rs:635-712 for static transforms; the area light is the
        diffuse emitter (pbrt-v2 semantics) on triangle meshes."""
        self._verify(STATE_WORLD_BLOCK, "Shape")
        if self.ctm[0] != self.ctm[1]:
            raise NotImplementedError("animated shapes (ActiveTransform end times) are not rendered on the device")
        o2w = self.ctm[0]
        shape = make_shape(name, o2w, o2w.inverse(), self.gs.reverse_orientation, ps)
        mtl = self.gs.create_material(ps)
        if self.gs.area_light:
            if self.gs.area_light != "diffuse":
                raise NotImplementedError(f"area light {self.gs.area_light!r}")
            f32 = np.float32
            L = self.gs.area_light_params.find_one_spectrum("L", (1.0, 1.0, 1.0))
            sc = self.gs.area_light_params.find_one_spectrum("scale", (1.0, 1.0, 1.0))
            light = DiffuseAreaLight(o2w, tuple(float(f32(a) * f32(b)) for a, b in zip(L, sc)))
            prim = Primitive.geometric_area_light(shape, mtl, light)
        else:
            prim = Primitive.geometric(shape, mtl)
        if self.current_instance is not None:
            self.instances[self.current_instance].append(prim)
        else:
            if prim.area_light is not None:
                self.lights.append(prim.area_light)
            self.primitives.append(prim)

    # instancing (main.rs:714-763)
    def object_begin(self, name):
        self._verify(STATE_WORLD_BLOCK, "ObjectBegin")
        self.attribute_begin()
        if self.current_instance is not None:
            raise RuntimeError("ObjectBegin called inside of instance definition")
        self.instances[name] = []
        self.definitions.pop(name, None)
        self.current_instance = name

    def object_end(self):
        self._verify(STATE_WORLD_BLOCK, "ObjectEnd")
        if self.current_instance is None:
            raise RuntimeError("ObjectEnd called outside of instance definition")
        self.current_instance = None
        self.attribute_end()

    def object_instance(self, name):
        """ObjectInstance (main.rs:735-763) placed as pbrt-v2 places it: a
        TransformedPrimitive (transformed.rs:14-59) over the definition's
        aggregate, its world-to-primitive transform the inverse of the
        current transform (the reference computes that transform but pushes
        the untransformed primitive, and cannot build the aggregate).  All
        instances of a definition share one device BVH.  A definition that
        holds area lights is copied out instead, shape by shape with the
        composed transform, since an emitter is sampled in world space."""
        self._verify(STATE_WORLD_BLOCK, "ObjectInstance")
        if name not in self.instances:
            print(f"Can't find object named {name}")
            return
        if not self.instances[name]:  # main.rs:741-743
            return
        if self.ctm[0] != self.ctm[1]:
            raise NotImplementedError("animated instances are not rendered on the device")
        inst = self.ctm[0]
        if all(p.area_light is None for p in self.instances[name]):
            defn = self.definitions.get(name)
            if defn is None:
                defn = self.definitions[name] = InstanceDefinition(list(self.instances[name]))
            self.primitives.append(Primitive.transformed(defn, inst.inverse()))
            return
        for p in self.instances[name]:
            s = p.shape
            moved = dataclasses.replace(s, object_to_world=inst * s.object_to_world)
            if p.area_light is not None:
                light = DiffuseAreaLight(inst * p.area_light.light_to_world, p.area_light.radiance)
                q = Primitive.geometric_area_light(moved, p.material, light)
                self.lights.append(light)
            else:
                q = Primitive.geometric(moved, p.material)
            self.primitives.append(q)

    def world_end(self) -> Frame:
        """main.rs:774-800: the frame is assembled (and rendered if asked);
        the state returns to the options block."""
        self._verify(STATE_WORLD_BLOCK, "WorldEnd")
        while self.pushed_gs:
            print("Missing end to pbrt_attribute_begin()")
            self.pushed_gs.pop()
            self.pushed_ctm.pop()
        while self.pushed_ctm:
            print("Missing end to pbrt_transform_begin()")
            self.pushed_ctm.pop()
        frame = self._make_frame()
        self.frames.append(frame)
        if self.render_on_world_end:
            frame.render()
        self.state = STATE_OPTIONS_BLOCK
        self.ctm = [Transform(), Transform()]
        self.active_transform_all()
        self.named_coordinate_systems.clear()
        lights, prims = self.lights, self.primitives
        self.lights, self.primitives = [], []
        del lights, prims
        return frame

    def _make_frame(self) -> Frame:
        fname, fps = self.filter
        filt = make_filter(fname, fps)
        film_name, ps = self.film
        if film_name != "image":
            raise NotImplementedError(f"film {film_name!r}")
        xres, yres = ps.find_one_int("xresolution", 640), ps.find_one_int("yresolution", 480)
        crop = ps.find_float("cropwindow")
        crop = tuple(float(c) for c in crop[:4]) if crop and len(crop) >= 4 else (0.0, 1.0, 0.0, 1.0)
        film = Film.image(xres, yres, filt, crop, ps.find_one_string("filename", ""))
        cam_name, cps = self.camera
        if cam_name != "perspective":
            raise NotImplementedError(f"camera {cam_name!r}: only the perspective camera exists")
        if self.camera_to_world[0] != self.camera_to_world[1]:
            raise NotImplementedError("animated cameras are not rendered on the device")
        frame_aspect = cps.find_one_float("frameaspectratio", xres / yres)
        if frame_aspect > 1.0:
            screen = (-frame_aspect, frame_aspect, -1.0, 1.0)
        else:
            screen = (-1.0, 1.0, -1.0 / frame_aspect, 1.0 / frame_aspect)
        sw = cps.find_float("screenwindow")
        if sw and len(sw) == 4:
            screen = tuple(float(c) for c in sw)
        sopen = cps.find_one_float("shutteropen", 0.0)
        sclose = cps.find_one_float("shutterclose", 1.0)
        camera = Camera.perspective(self.camera_to_world[0], screen, sopen, sclose, cps.find_one_float("lensradius", 0.0),
                                    cps.find_one_float("focaldistance", 1e30), cps.find_one_float("fov", 90.0), film)
        sname, sps = self.sampler
        if sname != "stratified":
            raise NotImplementedError(f"sampler {sname!r}: the device renders with the stratified sampler")
        x0, x1, y0, y1 = film.pixel_extent()
        sampler = StratifiedSampler.stratified(x0, x1, y0, y1, sps.find_one_int("xsamples", 2),
                                               sps.find_one_int("ysamples", 2), sps.find_one_bool("jitter", True),
                                               sopen, sclose)
        iname, _ = self.surface_integrator
        if iname not in ("directlighting", "whitted"):
            raise NotImplementedError(f"surface integrator {iname!r}")
        aname, aps = self.accelerator
        if aname != "bvh":
            raise NotImplementedError(f"accelerator {aname!r}: the device traverses the BVH")
        return Frame(self.primitives, self.lights, camera, sampler, aps.find_one_int("maxnodeprims", 4),
                     aps.find_one_string("splitmethod", "sah"), default_num_tasks(film.x_res, film.y_res))


# ------------------------------------------------------------------ parser
_TOKEN = re.compile(r'"[^"]*"|\[|\]|[^\s\[\]"]+')


def tokenize(text: str) -> list[str]:
    out = []
    for line in text.splitlines():
        # a '#' outside a string starts a comment
        parts, in_str = [], False
        for ch in line:
            if ch == '"':
                in_str = not in_str
            if ch == "#" and not in_str:
                break
            parts.append(ch)
        out += _TOKEN.findall("".join(parts))
    return out


def _number(tok: str) -> float:
    return float(tok)


class _Stream:
    def __init__(self, toks):
        self.t, self.i = toks, 0

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else None

    def next(self):
        tok = self.peek()
        if tok is None:
            raise SyntaxError("unexpected end of scene description")
        self.i += 1
        return tok

    def string(self) -> str:
        tok = self.next()
        if not (tok.startswith('"') and tok.endswith('"')):
            raise SyntaxError(f"expected a quoted string, got {tok!r}")
        return tok[1:-1]

    def numbers(self, n: int) -> list[float]:
        if self.peek() == "[":
            self.next()
            vals = []
            while self.peek() != "]":
                vals.append(_number(self.next()))
            self.next()
        else:
            vals = [_number(self.next()) for _ in range(n)]
        if len(vals) != n:
            raise SyntaxError(f"expected {n} numbers, got {len(vals)}")
        return vals

    def params(self) -> ParamSet:
        ps = ParamSet()
        while self.peek() is not None and self.peek().startswith('"'):
            decl = self.string().split()
            if len(decl) != 2:
                raise SyntaxError(f"bad parameter declaration {decl!r}")
            ty, name = decl
            if self.peek() == "[":
                self.next()
                raw = []
                while self.peek() != "]":
                    raw.append(self.next())
                self.next()
            else:
                raw = [self.next()]
            if ty in ("string", "texture"):
                vals = [r.strip('"') for r in raw]
            elif ty == "bool":
                vals = [r.strip('"') == "true" for r in raw]
            elif ty == "integer":
                vals = [int(float(r)) for r in raw]
            else:
                vals = [float(r) for r in raw]
            ps.add(ty, name, vals)
        return ps


def parse(text: str, api: Pbrt | None = None, base_dir: str = ".") -> Pbrt:
    """Runs a pbrt-v2 scene description through `api` (a new Pbrt if None)."""
    api = api or Pbrt()
    s = _Stream(tokenize(text))
    while s.peek() is not None:
        kw = s.next()
        if kw == "Identity":
            api.identity()
        elif kw == "Translate":
            api.translate(*s.numbers(3))
        elif kw == "Rotate":
            api.rotate(*s.numbers(4))
        elif kw == "Scale":
            api.scale(*s.numbers(3))
        elif kw == "LookAt":
            api.look_at(*s.numbers(9))
        elif kw in ("ConcatTransform", "Transform"):
            # scene files list the matrix column by column (pbrt-v2)
            xf = np.asarray(s.numbers(16), np.float32).reshape(4, 4).T.reshape(-1)
            (api.concat_transform if kw == "ConcatTransform" else api.transform)(xf)
        elif kw == "CoordinateSystem":
            api.coordinate_system(s.string())
        elif kw == "CoordSysTransform":
            api.coord_sys_transform(s.string())
        elif kw == "ActiveTransform":
            which = s.next()
            {"All": api.active_transform_all, "StartTime": api.active_transform_start_time,
             "EndTime": api.active_transform_end_time}[which]()
        elif kw == "TransformTimes":
            api.transform_times(*s.numbers(2))
        elif kw in ("PixelFilter", "Film", "Sampler", "Accelerator", "SurfaceIntegrator", "VolumeIntegrator",
                    "Renderer", "Camera", "Material", "MakeNamedMaterial", "LightSource", "AreaLightSource",
                    "Shape"):
            name = s.string()
            ps = s.params()
            {"PixelFilter": api.pixel_filter, "Film": api.film_, "Sampler": api.sampler_,
             "Accelerator": api.accelerator_, "SurfaceIntegrator": api.surface_integrator_,
             "VolumeIntegrator": api.volume_integrator_, "Renderer": api.renderer_, "Camera": api.camera_,
             "Material": api.material, "MakeNamedMaterial": api.make_named_material,
             "LightSource": api.light_source, "AreaLightSource": api.area_light_source,
             "Shape": api.shape}[kw](name, ps)
        elif kw == "Texture":
            name, ty, cls = s.string(), s.string(), s.string()
            api.texture(name, ty, cls, s.params())
        elif kw == "NamedMaterial":
            api.named_material(s.string())
        elif kw == "WorldBegin":
            api.world_begin()
        elif kw == "WorldEnd":
            api.world_end()
        elif kw == "AttributeBegin":
            api.attribute_begin()
        elif kw == "AttributeEnd":
            api.attribute_end()
        elif kw == "TransformBegin":
            api.transform_begin()
        elif kw == "TransformEnd":
            api.transform_end()
        elif kw == "ReverseOrientation":
            api.reverse_orientation()
        elif kw == "ObjectBegin":
            api.object_begin(s.string())
        elif kw == "ObjectEnd":
            api.object_end()
        elif kw == "ObjectInstance":
            api.object_instance(s.string())
        elif kw == "Include":
            path = os.path.join(base_dir, s.string())
            with open(path) as f:
                parse(f.read(), api, os.path.dirname(path))
        else:
            raise SyntaxError(f"unknown directive {kw!r}")
    return api


def parse_file(path: str, api: Pbrt | None = None) -> Pbrt:
    with open(path) as f:
        return parse(f.read(), api, os.path.dirname(os.path.abspath(path)))
