"""Scene ingestion: ParamSet, the scene-description API and the pbrt-v2
file parser build the same scene objects as the programmatic interface, and
the oracle renders them to the same image."""
import numpy as np
import pytest

from pbrt_rust_gb300 import api as A, generators as G
from pbrt_rust_gb300.scene import SceneDescription
from pbrt_rust_gb300.transform import Transform

# the plain render scene, written as a scene file (camera at (0, 1.5, -6)
# looking at the origin, fov 60, ground quad, two spheres, a point light
# and a 1x1 area light at y = 4 facing down)
SCENE = """
# camera and options
LookAt 0 1.5 -6   0 0 0   0 1 0
Camera "perspective" "float fov" [60] "float screenwindow" [-1 1 -1 1]
Film "image" "integer xresolution" [40] "integer yresolution" [32]
PixelFilter "box" "float xwidth" 0.5 "float ywidth" 0.5
Sampler "stratified" "integer xsamples" [2] "integer ysamples" [2] "bool jitter" "true"
SurfaceIntegrator "directlighting"
Accelerator "bvh" "integer maxnodeprims" [4] "string splitmethod" "sah"
WorldBegin
LightSource "point" "point from" [0 6 -2] "rgb I" [50 50 50]
AttributeBegin
  Material "matte" "rgb Kd" [0.5 0.5 0.5]
  Shape "trianglemesh" "integer indices" [0 1 2 0 2 3]
        "point P" [-10 0 -10  10 0 -10  10 0 10  -10 0 10]
AttributeEnd
Texture "red" "color" "constant" "rgb value" [0.7 0.2 0.2]
MakeNamedMaterial "shiny" "string type" "matte" "texture Kd" "red"
AttributeBegin
  NamedMaterial "shiny"
  Translate 0.5 0.4 0.2
  Shape "sphere" "float radius" 0.4
AttributeEnd
ObjectBegin "ball"
  Material "matte" "rgb Kd" [0.2 0.6 0.3]
  Shape "sphere" "float radius" 0.25
ObjectEnd
AttributeBegin
  Translate -1 0.3 1
  ObjectInstance "ball"
AttributeEnd
AttributeBegin
  AreaLightSource "diffuse" "rgb L" [10 10 10]
  Material "matte" "rgb Kd" [0 0 0]
  Shape "trianglemesh" "integer indices" [0 2 1 0 3 2]
        "point P" [-0.5 4 -0.5  0.5 4 -0.5  0.5 4 0.5  -0.5 4 0.5]
AttributeEnd
WorldEnd
"""


def test_paramset_lookups():
    ps = A.ParamSet()
    ps.add("float", "radius", [2.5])
    ps.add("integer", "indices", [0, 1, 2])
    ps.add("color", "Kd", [0.1, 0.2, 0.3])
    ps.add("bool", "jitter", [False])
    assert ps.find_one_float("radius", 1.0) == 2.5 and ps.find_one_float("missing", 1.0) == 1.0
    assert ps.find_one_int("radius", 7) == 7  # wrong type: the default (params.rs:87-94)
    assert ps.find_int("indices") == [0, 1, 2]
    assert ps.find_one_spectrum("Kd", (0, 0, 0)) == pytest.approx((0.1, 0.2, 0.3))
    assert ps.find_one_bool("jitter", True) is False


def test_scene_file_builds_the_programmatic_scene():
    frame = A.parse(SCENE).frames[0]
    assert len(frame.primitives) == 4 and len(frame.lights) == 2
    cam = frame.camera
    want = Transform.look_at((0.0, 1.5, -6.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0)).inverse()
    assert cam.camera_to_world == want and cam.fov == 60.0
    assert (cam.film.x_res, cam.film.y_res) == (40, 32)
    s = frame.sampler
    assert (s.x_samples, s.y_samples, s.jitter, s.x_end, s.y_end) == (2, 2, True, 40, 32)
    ground, sphere, inst, quad = frame.primitives
    assert ground.material.kd == pytest.approx((0.5, 0.5, 0.5))
    assert sphere.material.kd == pytest.approx((0.7, 0.2, 0.2)) and sphere.shape.radius == 0.4
    assert sphere.shape.object_to_world == Transform.translate((0.5, 0.4, 0.2))
    assert inst.shape.object_to_world == Transform.translate((-1.0, 0.3, 1.0))  # placed by the instance
    assert quad.area_light is not None and quad.area_light.radiance == (10.0, 10.0, 10.0)
    assert frame.lights[0].light_to_world == Transform.translate((0.0, 6.0, -2.0))


def test_scene_file_renders_like_the_programmatic_scene(oracle):
    frame = A.parse(SCENE).frames[0]
    img = oracle.render(SceneDescription(frame.primitives, frame.lights, frame.max_prims, frame.split_method),
                        frame.camera, frame.sampler, frame.num_tasks)
    assert img.max() > 0.1 and img.shape == (32, 40, 3)
    # the same scene built through the Python interface
    prims, lights, cam, smp = G.c1_scene(res=40, n_spheres=0)
    assert frame.primitives[0].shape.points.tolist() == prims[0].shape.points.tolist()


def test_transforms_compose_like_the_reference():
    p = A.Pbrt()
    p.translate(1, 2, 3)
    p.scale(2, 2, 2)
    p.rotate(90, 0, 0, 1)
    t = Transform.translate((1, 2, 3)) * Transform.scale(2, 2, 2) * Transform.rotate(90, (0, 0, 1))
    assert p.ctm[0] == t and p.ctm[1] == t
    p.active_transform_end_time()
    p.translate(5, 0, 0)
    assert p.ctm[0] == t and p.ctm[1] != t


def test_matrix_directives_and_coordinate_systems():
    p = A.parse("ConcatTransform [1 0 0 0  0 1 0 0  0 0 1 0  4 5 6 1] CoordinateSystem \"a\" Identity "
                "CoordSysTransform \"a\"")
    assert p.ctm[0] == Transform.translate((4.0, 5.0, 6.0))


def test_unsupported_directives_fail_loudly():
    with pytest.raises(NotImplementedError):
        A.parse('WorldBegin Shape "cone" WorldEnd')
    with pytest.raises(NotImplementedError):
        A.parse('Sampler "lowdiscrepancy" WorldBegin WorldEnd')
    with pytest.raises(SyntaxError):
        A.parse('Frobnicate 1 2 3')
    with pytest.raises(RuntimeError):
        A.parse('Shape "sphere"')  # outside the world block
