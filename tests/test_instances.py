"""TransformedPrimitive instances (src/primitive/transformed.rs:14-73) in
the oracle and at the C ABI, without a GPU.

An instance traces the primitive-space ray w2p(ray) through its
definition's aggregate and reports the id (first id of the instance) +
(refined index inside the definition)."""
import ctypes as C

import numpy as np
import pytest

from pbrt_rust_gb300 import abi, generators as G
from pbrt_rust_gb300.scene import InstanceDefinition, MatteMaterial, Primitive, SceneDescription, Shape
from pbrt_rust_gb300.transform import Transform

INVALID_ARGUMENT, UNSUPPORTED = 1, 4  # PbrtStatus

def tri_mesh(pts, idx=None):
    pts = np.asarray(pts, np.float32)
    idx = np.arange(len(pts), dtype=np.uint32) if idx is None else np.asarray(idx, np.uint32)
    return Shape.triangle_mesh(Transform(), None, False, idx, pts)


def ray(o, d, tmin=0.0, tmax=np.inf):
    r = np.zeros(8, np.float32)
    r[0:3], r[3], r[4:7], r[7] = o, tmin, d, tmax
    return r.reshape(1, 8)


def test_translated_instance_known_answer(oracle):
    """A unit right triangle in the z = 0 plane, instanced 5 units along
    +x: the ray (5.25, 0.25, -1) + t (0, 0, 1) hits it at t = 1 with the
    barycentrics of the untranslated triangle."""
    defn = InstanceDefinition([Primitive.simple(tri_mesh([(0, 0, 0), (1, 0, 0), (0, 1, 0)]))])
    inst = Primitive.transformed(defn, Transform.translate((5.0, 0.0, 0.0)).inverse())
    o = oracle.OracleBVH([inst])
    h = o.intersect(ray((5.25, 0.25, -1.0), (0.0, 0.0, 1.0)))[0]
    plain = oracle.OracleBVH([Primitive.simple(tri_mesh([(0, 0, 0), (1, 0, 0), (0, 1, 0)]))])
    want = plain.intersect(ray((0.25, 0.25, -1.0), (0.0, 0.0, 1.0)))[0]
    assert h["prim"] == 0 and h["t"] == np.float32(1.0)
    assert (h["b1"], h["b2"]) == (want["b1"], want["b2"])
    assert o.intersect(ray((0.25, 0.25, -1.0), (0.0, 0.0, 1.0)))[0]["prim"] == -1
    assert o.intersect_p(ray((5.25, 0.25, -1.0), (0.0, 0.0, 1.0)))[0] == 1
    # maxt below the hit: no hit
    assert o.intersect(ray((5.25, 0.25, -1.0), (0.0, 0.0, 1.0), tmax=0.5))[0]["prim"] == -1


def test_instance_ids_count_the_definition_out(oracle):
    """Scene = [mesh of 3 triangles, instance of a 2-triangle definition,
    sphere]: the instance takes ids 3 and 4, the sphere id 5."""
    mesh = tri_mesh([(0, 0, 0), (1, 0, 0), (0, 1, 0), (2, 0, 0), (3, 0, 0), (2, 1, 0), (4, 0, 0), (5, 0, 0),
                     (4, 1, 0)])
    two = tri_mesh([(0, 0, 0), (1, 0, 0), (0, 1, 0), (2, 0, 0), (3, 0, 0), (2, 1, 0)])
    defn = InstanceDefinition([Primitive.simple(two)])
    inst = Primitive.transformed(defn, Transform.translate((0.0, 5.0, 0.0)).inverse())
    sph = Shape.sphere(Transform.translate((10.0, 0.0, 0.0)), None, False, 0.5, -0.5, 0.5, 360.0)
    prims = [Primitive.simple(mesh), inst, Primitive.simple(sph)]
    assert SceneDescription(prims, []).num_ids() == 6
    o = oracle.OracleBVH(prims)
    rays = np.concatenate([ray((0.2, 0.2, -1), (0, 0, 1)), ray((2.2, 5.2, -1), (0, 0, 1)),
                           ray((0.2, 5.2, -1), (0, 0, 1)), ray((10.0, 0.0, -3), (0, 0, 1))])
    assert list(o.intersect(rays)["prim"]) == [0, 4, 3, 5]
    assert o.num_primitives() == 5  # mesh triangles + one instance + one sphere


def test_instanced_scene_agrees_with_its_copied_out_twin(oracle):
    """The same forest with every instance copied out (composed transforms)
    is a different f32 computation; hits agree up to rounding."""
    prims, _, _, _, flat = G.instanced_forest(n_instances=24, tris_per_tree=300, seed=3)
    a, b = oracle.OracleBVH(prims), oracle.OracleBVH(flat)
    rays = G.rays_toward_center(G.PCG32(2), 1 << 13, radius=14.0, target=4.0)
    ha, hb = a.intersect(rays), b.intersect(rays)
    assert (ha["prim"] >= 0).sum() > 2000
    same = ha["prim"] == hb["prim"]
    assert same.mean() > 0.995
    both = same & (ha["prim"] >= 0)
    assert np.allclose(ha["t"][both], hb["t"][both], rtol=1e-4, atol=1e-5)
    assert np.mean(a.intersect_p(rays) == b.intersect_p(rays)) > 0.995


def test_instance_bound_is_the_transformed_definition_bound(oracle):
    """transformed.rs:62-65: world bound = primitive-to-world applied to the
    definition's bound (the bbox transform of transform.rs:248-264)."""
    defn = InstanceDefinition([Primitive.simple(tri_mesh([(0, 0, 0), (1, 0, 0), (0, 1, 0)]))])
    i2w = Transform.translate((1.0, 2.0, 3.0)) * Transform.scale(2.0, 2.0, 2.0)
    o = oracle.OracleBVH([Primitive.transformed(defn, i2w.inverse())])
    lo, hi = o.world_bound()
    assert np.array_equal(lo, np.float32([1, 2, 3])) and np.array_equal(hi, np.float32([3, 4, 3]))


def _desc_status(desc):
    lib = abi.load()
    h = C.c_void_p()
    st = lib.pbrtgpu_bvh_create_desc(C.byref(desc.desc), C.byref(h))
    if st == 0:
        lib.pbrtgpu_bvh_destroy(h)
    return st


def test_c_abi_builds_and_rejects_instances():
    """pbrtgpu_bvh_create_desc builds (host build, no device needed) and
    refuses nested instances, emitters inside definitions, empty
    definitions and out-of-range definition indices."""
    prims, _, _, _, _ = G.instanced_forest(n_instances=8, tris_per_tree=100, seed=1)
    desc = SceneDescription(prims, [], aggregate_only=True)
    assert _desc_status(desc) == 0
    inner = InstanceDefinition([Primitive.simple(tri_mesh([(0, 0, 0), (1, 0, 0), (0, 1, 0)]))])
    with pytest.raises(ValueError):
        Primitive.transformed(InstanceDefinition([Primitive.transformed(inner, Transform())]), Transform())
    with pytest.raises(ValueError):
        Primitive.transformed(InstanceDefinition([]), Transform())
    # the same checks at the ABI, past the Python front end
    d = SceneDescription([Primitive.transformed(inner, Transform())], [], aggregate_only=True)
    d.def_shapes[0][0].kind = abi.SHAPE_INSTANCE
    d.def_shapes[0][0].instance = 0
    assert _desc_status(d) == UNSUPPORTED
    d = SceneDescription([Primitive.transformed(inner, Transform())], [], aggregate_only=True)
    d.def_shapes[0][0].area_light = 0
    assert _desc_status(d) == UNSUPPORTED
    d = SceneDescription([Primitive.transformed(inner, Transform())], [], aggregate_only=True)
    d.instance_descs[0].n_shapes = 0
    assert _desc_status(d) == INVALID_ARGUMENT
    d = SceneDescription([Primitive.transformed(inner, Transform())], [], aggregate_only=True)
    d.shapes[0].instance = 1
    assert _desc_status(d) == INVALID_ARGUMENT


def test_scene_file_instances_share_one_definition():
    """ObjectBegin / ObjectInstance in a scene file: every instance of a
    name refers to the same definition; a definition with an emitter is
    copied out instead."""
    from pbrt_rust_gb300.api import parse
    text = """
    LookAt 0 2 -8  0 0 0  0 1 0
    Camera "perspective" "float fov" [45]
    Film "image" "integer xresolution" [16] "integer yresolution" [16]
    Sampler "stratified" "integer xsamples" [1] "integer ysamples" [1]
    WorldBegin
    ObjectBegin "box"
      Shape "trianglemesh" "integer indices" [0 1 2 0 2 3] "point P" [-1 0 -1 1 0 -1 1 0 1 -1 0 1]
      Shape "sphere" "float radius" [0.5]
    ObjectEnd
    ObjectBegin "lamp"
      AreaLightSource "diffuse" "rgb L" [4 4 4]
      Shape "trianglemesh" "integer indices" [0 1 2] "point P" [0 3 0 1 3 0 0 3 1]
    ObjectEnd
    AttributeBegin
      Translate 2 0 0
      ObjectInstance "box"
    AttributeEnd
    AttributeBegin
      Translate -2 0 0
      Rotate 30 0 1 0
      ObjectInstance "box"
    AttributeEnd
    ObjectInstance "lamp"
    WorldEnd
    """
    frame = parse(text).frames[-1]
    inst = [p for p in frame.primitives if p.shape.kind == abi.SHAPE_INSTANCE]
    assert len(inst) == 2 and inst[0].shape.definition is inst[1].shape.definition
    assert len(inst[0].shape.definition.prims) == 2
    assert len(frame.lights) == 1  # the lamp was copied out
    desc = SceneDescription(frame.primitives, frame.lights)
    assert desc.desc.n_instances == 1 and desc.num_ids() == 2 * 3 + 1


def test_instancing_keeps_one_copy_of_each_definition():
    """Instances share the definition's BVH: the scene's own tree has one
    primitive per instance, against every triangle once copied out."""
    from pbrt_rust_gb300.gpu import GpuBVHAccel
    prims, _, _, _, flat = G.instanced_forest(n_instances=64, tris_per_tree=2000, seed=1)
    inst, copied = GpuBVHAccel(prims), GpuBVHAccel(flat)
    assert inst.num_primitives() == 2 + 64 + 2  # ground, instances, lamp
    assert copied.num_primitives() == 2 + 32 * (2000 + 2) + 32 * (1 + 2) + 2
    assert copied.num_nodes() > 100 * inst.num_nodes()
    assert copied.device_bytes() > 25 * inst.device_bytes()
