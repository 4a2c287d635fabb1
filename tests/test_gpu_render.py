"""GPU parity of the render wavefront against the CPU oracle.

Images rendered with identical sample streams must match per pixel within
1e-4 absolute in linear RGB.  Triangle-only scenes come out bit-identical;
sphere normals go through acosf/sinf, whose CUDA and glibc results may
differ in the last bit, which moves a pixel by ~1e-7.
"""
import numpy as np
import pytest

from pbrt_rust_gb300 import generators as G
from pbrt_rust_gb300.gpu import GpuSamplerRenderer, GpuScene
from pbrt_rust_gb300.scene import (Camera, Film, Filter, MatteMaterial, SceneDescription, StratifiedSampler,
                                   default_num_tasks)

pytestmark = pytest.mark.gpu
TOL = 1e-4


def render_both(oracle, prims, lights, cam, smp, num_tasks=None):
    nt = num_tasks or default_num_tasks(cam.film.x_res, cam.film.y_res)
    scene = GpuScene(prims, lights, 4, "sah")
    gpu = GpuSamplerRenderer(smp, cam, num_tasks=nt).render(scene)
    ref = oracle.render(SceneDescription(prims, lights, 4, "sah"), cam, smp, nt)
    return gpu, ref


def assert_image_close(gpu, ref):
    assert gpu.shape == ref.shape
    assert np.isfinite(gpu).all()
    diff = np.abs(gpu - ref)
    assert diff.max() <= TOL, (diff.max(), np.unravel_index(diff.argmax(), diff.shape))
    assert ref.max() > 0.1  # the image is not trivially black


@pytest.fixture(params=["plain", "packet"])
def render_kernel(request):
    """The render's camera and shadow rays through the per-lane walk and
    through the warp-cooperative one: the same images."""
    from pbrt_rust_gb300 import abi
    before = abi.get_trace_config()
    abi.set_trace_config(render_kernel=request.param)
    yield request.param
    abi.set_trace_config(**before)


@pytest.mark.parametrize("res", [64, 512])
def test_c1_render_matches_oracle(oracle, res, render_kernel):
    """The plain render (spheres, ground, point + area light, 2x2 strata)."""
    prims, lights, cam, smp = G.c1_scene(res=res)
    gpu, ref = render_both(oracle, prims, lights, cam, smp)
    assert_image_close(gpu, ref)


def test_triangle_scene_is_bit_exact(oracle, render_kernel):
    """Without spheres every step is exact IEEE f32: the images are equal."""
    prims, lights, cam, smp = G.c1_scene(res=96, n_spheres=0)
    prims += G.ray_soup(500, 1, seed=5)[0]
    gpu, ref = render_both(oracle, prims, lights, cam, smp)
    assert np.array_equal(gpu.view(np.uint32), ref.view(np.uint32))


def thin_lens_case(res=72, xs=3, ys=3):
    """A triangle-only C1 scene through a thin-lens camera (lens radius
    0.08, focal distance 5.5): the sampler's general path with its lens and
    time strata and their shuffles (projective.rs:79-96)."""
    prims, lights, cam0, _ = G.c1_scene(res=res, n_spheres=0)
    prims += G.ray_soup(300, 1, seed=7)[0]
    cam = Camera.perspective(cam0.camera_to_world, cam0.screen_window, 0.0, 1.0, 0.08, 5.5, cam0.fov, cam0.film)
    smp = StratifiedSampler.stratified(0, res, 0, res, xs, ys, True, 0.0, 1.0)
    return prims, lights, cam, smp


@pytest.mark.parametrize("xs,ys", [(3, 3), (2, 2), (1, 1)])
def test_thin_lens_camera_is_bit_exact(oracle, xs, ys):
    """Odd and even sample counts per pixel through the thin lens; without
    spheres every step is exact f32, so the images are equal."""
    prims, lights, cam, smp = thin_lens_case(xs=xs, ys=ys)
    gpu, ref = render_both(oracle, prims, lights, cam, smp)
    assert np.array_equal(gpu.view(np.uint32), ref.view(np.uint32))
    pin = render_both(oracle, *thin_lens_case(xs=xs, ys=ys)[:2],
                      Camera.perspective(cam.camera_to_world, cam.screen_window, 0.0, 1.0, 0.0, 1e30, cam.fov,
                                         cam.film), smp)[1]
    assert not np.array_equal(ref, pin)  # the lens changes the image


@pytest.mark.parametrize("xs,ys,jitter,tasks", [(1, 1, True, 8), (4, 4, True, 3), (3, 2, False, 5), (2, 2, True, 1)])
def test_sampler_variants(oracle, xs, ys, jitter, tasks):
    prims, lights, cam, _ = G.c1_scene(res=80)
    smp = StratifiedSampler.stratified(0, 80, 0, 80, xs, ys, jitter, 0.0, 1.0)
    gpu, ref = render_both(oracle, prims, lights, cam, smp, tasks)
    assert_image_close(gpu, ref)


def test_non_square_crop_and_wide_filter(oracle):
    """Aspect != 1, a crop window, a sampler window smaller than the film and
    a box filter of width 1 (each sample lands on up to 4 pixels)."""
    prims, lights, cam0, _ = G.c1_scene(res=64)
    film = Film.image(120, 72, Filter.mean(1.0, 1.0), (0.1, 0.9, 0.05, 1.0))
    cam = Camera.perspective(cam0.camera_to_world, (-120 / 72, 120 / 72, -1.0, 1.0), 0.0, 1.0, 0.0, 1e30, 60.0, film)
    smp = StratifiedSampler.stratified(5, 115, 0, 70, 2, 2, True, 0.0, 1.0)
    gpu, ref = render_both(oracle, prims, lights, cam, smp, 6)
    assert_image_close(gpu, ref)


def test_render_into_device_tensor(oracle):
    import torch
    prims, lights, cam, smp = G.c1_scene(res=64)
    scene = GpuScene(prims, lights)
    r = GpuSamplerRenderer(smp, cam)
    out = torch.zeros((64, 64, 3), dtype=torch.float32, device="cuda")
    r.render(scene, out=out)
    torch.cuda.synchronize()
    host = r.render(scene)
    assert np.array_equal(out.cpu().numpy(), host)


def test_repeat_render_is_deterministic():
    prims, lights, cam, smp = G.c1_scene(res=128)
    scene = GpuScene(prims, lights)
    r = GpuSamplerRenderer(smp, cam)
    a = r.render(scene)
    b = r.render(scene)
    assert np.array_equal(a, b)


def test_task_shards_sum_to_the_frame():
    """pbrtgpu_render_tasks over disjoint task ranges: the images add up to
    pbrtgpu_render's frame bit for bit (a frame sharded over ranks)."""
    from pbrt_rust_gb300.shard import task_range
    prims, lights, cam, smp = G.c1_scene(res=72)
    scene = GpuScene(prims, lights)
    r = GpuSamplerRenderer(smp, cam)
    full = r.render(scene)
    for world in (2, 3):
        acc = np.zeros_like(full)
        for rank in range(world):
            part = r.render(scene, tasks=task_range(r.num_tasks, world, rank))
            assert part.max() > 0.0
            acc += part
        assert np.array_equal(acc.view(np.uint32), full.view(np.uint32))
    empty = r.render(scene, tasks=(2, 2))
    assert not empty.any()


@pytest.mark.parametrize("filt", [Filter.triangle(2.0, 1.5), Filter.gaussian(2.0, 2.0, 2.0),
                                  Filter.mitchell(2.0, 2.0, 1.0 / 3.0, 1.0 / 3.0), Filter.lanczos(3.0, 2.5, 3.0)],
                         ids=lambda f: f.kind)
def test_filters_match_oracle(oracle, filt):
    """Wide, negative-lobed and separable filters: every pixel gathers the
    samples of its neighbours with the table weights."""
    prims, lights, cam, _ = G.c1_scene(res=56)
    cam = Camera.perspective(cam.camera_to_world, cam.screen_window, 0.0, 1.0, 0.0, 1e30, cam.fov,
                             Film.image(56, 40, filt))
    smp = StratifiedSampler.stratified(0, 56, 0, 40, 2, 2, True, 0.0, 1.0)
    gpu, ref = render_both(oracle, prims, lights, cam, smp)
    assert_image_close(gpu, ref)
    prims, lights, cam, _ = G.c1_scene(res=48, n_spheres=0)
    cam = Camera.perspective(cam.camera_to_world, cam.screen_window, 0.0, 1.0, 0.0, 1e30, cam.fov,
                             Film.image(48, 48, filt))
    smp = StratifiedSampler.stratified(0, 48, 0, 48, 2, 2, True, 0.0, 1.0)
    gpu, ref = render_both(oracle, prims, lights, cam, smp)
    assert np.array_equal(gpu.view(np.uint32), ref.view(np.uint32))


def test_scene_file_renders_on_the_device(oracle, tmp_path):
    """A pbrt-v2 scene file through the API (pbrt_rust_gb300.api) renders on
    the device as the oracle renders the parsed scene, and its film file is
    written."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from test_api import SCENE

    from pbrt_rust_gb300 import api as A
    text = SCENE.replace('Film "image"', f'Film "image" "string filename" "{tmp_path / "out.png"}"')
    frame = A.parse(text).frames[0]
    gpu = frame.render()
    ref = oracle.render(SceneDescription(frame.primitives, frame.lights, frame.max_prims, frame.split_method),
                        frame.camera, frame.sampler, frame.num_tasks)
    assert_image_close(gpu, ref)
    assert (tmp_path / "out.png").stat().st_size > 40 * 32 * 3


def test_disk_and_cylinder_scene_matches_oracle(oracle):
    """Shading of disks (the transformed +-z normal, disk.rs:125-129) and
    cylinders (helpers.rs:17-43) in the plain render scene."""
    from pbrt_rust_gb300.scene import Primitive, Shape
    from pbrt_rust_gb300.transform import Transform
    prims, lights, cam, smp = G.c1_scene(res=64, n_spheres=0)
    for i in range(6):
        t = Transform.translate((i - 2.5, 0.6, (i % 3) * 0.8 - 0.8)) * Transform.rotate(-90.0 + 25.0 * i, (1, 0, 0))
        s = (Shape.disk(t, None, i % 4 == 1, 0.0, 0.45, 0.1, 360.0) if i % 2
             else Shape.cylinder(t, None, False, 0.3, -0.4, 0.4, 360.0))
        prims.append(Primitive.geometric(s, MatteMaterial((0.3 + 0.1 * i, 0.5, 0.7 - 0.1 * i))))
    gpu, ref = render_both(oracle, prims, lights, cam, smp)
    assert_image_close(gpu, ref)


def test_oren_nayar_triangle_scene_is_bit_exact(oracle):
    """Matte with sigma > 0 is Oren-Nayar (matte.rs:42-47, orennayar.rs):
    its frame comes from dp/du; triangle-only scenes stay exact IEEE f32."""
    prims, lights, cam, smp = G.c1_scene(res=96, n_spheres=0)
    soup = G.ray_soup(400, 1, seed=6)[0]
    for i, p in enumerate(soup):
        p.material = MatteMaterial((0.3 + 0.001 * i, 0.6, 0.4), sigma=(5.0, 20.0, 60.0, 90.0, 150.0)[i % 5])
    prims[0].material = MatteMaterial((0.5, 0.5, 0.5), sigma=35.0)
    prims += soup
    gpu, ref = render_both(oracle, prims, lights, cam, smp)
    assert np.array_equal(gpu.view(np.uint32), ref.view(np.uint32))
    assert ref.max() > 0.1


def test_oren_nayar_quadrics_and_instances_match_oracle(oracle):
    """dp/du of spheres, disks (with the phi_max / 2 pi factor of
    disk.rs:114-116) and cylinders, and of instance hits moved by
    primitive-to-world (transformed.rs:48)."""
    from pbrt_rust_gb300.scene import InstanceDefinition, Primitive, Shape
    from pbrt_rust_gb300.transform import Transform
    prims, lights, cam, smp = G.c1_scene(res=64, n_spheres=10)
    for i, p in enumerate(prims[1:11]):
        p.material = MatteMaterial(p.material.kd, sigma=15.0 + 7.0 * i)
    for i in range(4):
        t = Transform.translate((i - 1.5, 0.6, -1.0)) * Transform.rotate(-90.0 + 30.0 * i, (1, 0, 0))
        s = (Shape.disk(t, None, False, 0.0, 0.45, 0.1, 300.0) if i % 2
             else Shape.cylinder(t, None, False, 0.3, -0.4, 0.4, 360.0))
        prims.append(Primitive.geometric(s, MatteMaterial((0.6, 0.4, 0.3), sigma=40.0)))
    defn = InstanceDefinition([
        Primitive.geometric(Shape.sphere(Transform(), None, False, 0.3, -0.3, 0.3, 360.0), MatteMaterial((0.7,) * 3, 25.0)),
        Primitive.geometric(Shape.disk(Transform.translate((0.0, 0.0, -0.3)), None, False, 0.0, 0.4, 0.0, 360.0),
                            MatteMaterial((0.2, 0.7, 0.3), 50.0))])
    for k in range(3):
        i2w = Transform.translate((-1.0 + k, 1.6, 1.0)) * Transform.rotate(40.0 * k, (0, 1, 0)) * Transform.scale(1.3, 1.3, 1.3)
        prims.append(Primitive.transformed(defn, i2w.inverse()))
    gpu, ref = render_both(oracle, prims, lights, cam, smp)
    assert_image_close(gpu, ref)
