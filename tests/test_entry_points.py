"""Reference entry points with parity tests of their own, through the C ABI on the GPU:
render_with_lights_and_environment_hdr_image (renderer.rs:588-609; area lights before the
environment in each bounce, camera.rs:1782-1805), render_with_light_connections
(renderer.rs:771-786; the reference's own test camera.rs:5636-5684 and
raytracing.rs:1730-1776), f32 denoising AOVs (camera.rs:4187-4244) and their independence
of the schedule (camera.rs:5235-5265's tiled == untiled), render_scene with the four
SurfaceRayMaterialModes (scene.rs:30-72, 1517-1547; renderer.rs:309-371), the
explicit tone mapping render (raytracing.rs:1504-1523) and the two-leaf traversal
statistics (bvh.rs:666-709)."""
import numpy as np
import pytest

import oracle
from gartus_gb300 import abi, scenes
from gartus_gb300.raytracing import (TONE_MAP_REINHARD, EnvironmentLight, PathTracer, RayCamera, RayMaterial,
                                     RayScene, SamplingTargetList, SurfaceMaterial, SurfaceRayMaterialMode,
                                     SurfaceScene, ToneMap)
from tests.divergence import assert_explained
from tests.helpers import rel_err
from tests.test_reference_known_answers import two_leaf_scene

pytestmark = pytest.mark.gpu

SCHEDULES = ["wavefront", "auto", "persistent"]


def _oracle(scene, cam, lights=None, env=None, precision=1, aovs=False):
    o = oracle.OracleScene.from_ray_scene(scene)
    la = lights.to_array() if lights is not None else None
    return o.render(cam.desc(), la, env, precision=precision, threads=8, aovs=aovs)


def _lit_room():
    """A box room with a ceiling quad light, a glass sphere, a metal sphere and a GGX block
    under an 8-bit environment seen through an opening in the roof."""
    scene = RayScene()
    white = scene.add_material(RayMaterial.lambertian((0.73, 0.73, 0.73)))
    red = scene.add_material(RayMaterial.lambertian((0.65, 0.05, 0.05)))
    light = scene.add_material(RayMaterial.diffuse_light((12.0, 12.0, 12.0)))
    glass = scene.add_material(RayMaterial.dielectric(1.5))
    metal = scene.add_material(RayMaterial.metal((0.8, 0.7, 0.6), 0.1))
    ggx = scene.add_material(RayMaterial.ggx_microfacet((0.8, 0.8, 0.8), 0.3))
    scene.add_quad((-3, -1, -6), (6, 0, 0), (0, 0, 6), white)   # floor
    scene.add_quad((-3, -1, -6), (0, 4, 0), (0, 0, 6), red)     # left wall
    scene.add_quad((-3, -1, -6), (6, 0, 0), (0, 4, 0), white)   # back wall
    scene.add_quad((-3, 3, -6), (3, 0, 0), (0, 0, 6), white)    # half a roof: the sky shows
    scene.add_quad((-1, 2.99, -4), (1.5, 0, 0), (0, 0, 1.5), light)
    scene.add_sphere((0.8, -0.2, -3.5), 0.8, glass)
    scene.add_sphere((-1.5, -0.4, -4.0), 0.6, metal)
    scene.add_quad((1.6, -1, -5), (0.8, 0, 0), (0, 1.5, 0), ggx)
    lights = SamplingTargetList()
    lights.add_quad((-1, 2.99, -4), (1.5, 0, 0), (0, 0, 1.5))
    rng = np.random.default_rng(11)
    env = EnvironmentLight(rng.integers(0, 256, size=(8, 16, 3), dtype=np.uint8))
    cam = (RayCamera(36, 1.0).with_samples_per_pixel(4).with_max_depth(12).with_look_at((0, 1, 2), (0, 0.5, -4))
           .with_vertical_fov(60.0).with_rng_seed(7))
    return scene, lights, env, cam


@pytest.mark.parametrize("mode", ["nee", "mixture"])
@pytest.mark.parametrize("schedule", SCHEDULES)
def test_lights_and_environment_match_oracle(gpu_context, mode, schedule):
    scene, lights, env, cam = _lit_room()
    if mode == "nee":
        cam = cam.with_direct_lighting_mode(abi.GT_DIRECT_NEXT_EVENT_ESTIMATION)
    pt = PathTracer(cam, precision="f64", context=gpu_context, schedule=schedule)
    img = pt.render_with_lights_and_environment_hdr_image(scene, lights, env, want64=True)
    ref, acc = _oracle(scene, cam, lights, env)
    np.testing.assert_array_equal(img.accepted, acc)
    err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
    print(f"{mode}/{schedule}: f64 max relative error {err.max():.3e}")
    assert err.max() <= 1e-9
    assert (ref.max(axis=2) > 0).mean() > 0.9
    img32 = PathTracer(cam, context=gpu_context, schedule=schedule).render_with_lights_and_environment_hdr_image(
        scene, lights, env)
    ref32, _ = _oracle(scene, cam, lights, env, precision=0)
    assert_explained(f"lights + environment {mode}/{schedule}", scene, cam, img32.pixels, ref, ref32, lights, env)


def test_light_connections_equal_next_event_render(gpu_context):
    # camera.rs:5636-5684: a current-path-continuation camera's light-connection render
    # equals its next-event render, for the explicit and the automatic target lists.
    scene = RayScene()
    diffuse = scene.add_material(RayMaterial.lambertian((0.7, 0.7, 0.7)))
    light = scene.add_material(RayMaterial.diffuse_light((4.0, 4.0, 4.0)))
    scene.add_sphere((0.0, 0.0, -1.0), 0.5, diffuse)
    scene.add_quad((-0.5, 1.0, -1.5), (1.0, 0.0, 0.0), (0.0, 0.0, 1.0), light)
    lights = SamplingTargetList()
    lights.add_quad((-0.5, 1.0, -1.5), (1.0, 0.0, 0.0), (0.0, 0.0, 1.0))
    cam = (RayCamera(16, 1.0).with_samples_per_pixel(4).with_max_depth(4).with_background((0.0, 0.0, 0.0))
           .with_direct_lighting_mode(abi.GT_DIRECT_CURRENT_PATH_CONTINUATION).with_rng_seed(321))
    nee = cam.with_direct_lighting_mode(abi.GT_DIRECT_NEXT_EVENT_ESTIMATION)
    for precision in ("f64", "f32"):
        expected = PathTracer(nee, precision=precision, context=gpu_context).render_with_lights_hdr_image(
            scene, lights, want64=precision == "f64")
        pt = PathTracer(cam, precision=precision, context=gpu_context)
        actual = pt.render_with_light_connections_hdr_image(scene, lights, want64=precision == "f64")
        auto = pt.render_ray_scene_with_light_connections_hdr_image(scene, want64=precision == "f64")
        np.testing.assert_array_equal(actual.pixels, expected.pixels)
        np.testing.assert_array_equal(auto.pixels, expected.pixels)
        if precision == "f64":
            ref, acc = _oracle(scene, nee, lights)
            assert rel_err(actual.pixels64, ref, floor=1e-12).max() <= 1e-9
            np.testing.assert_array_equal(actual.accepted, acc)
    assert actual.pixels.max() > 0


def test_f32_aovs_match_oracle_and_schedules(gpu_context):
    # The denoiser's inputs are the f32 AOVs: first-hit albedo and normal of every sample,
    # averaged.  Against the f64 oracle they agree to f32 rounding except on pixels where a
    # sample's primary ray meets a silhouette or an edge within f32 rounding (counted).
    # Like the reference's tiled and untiled AOV renders, every schedule gives the same AOVs.
    scene = scenes.final_scene_ray_scene()
    cam = scenes.final_scene_camera(96, 4)
    out = {}
    for schedule in SCHEDULES:
        out[schedule] = PathTracer(cam, context=gpu_context, schedule=schedule).render_denoising_aovs(scene)
    for schedule in SCHEDULES[1:]:
        np.testing.assert_array_equal(out[schedule].albedo_linear, out["wavefront"].albedo_linear)
        np.testing.assert_array_equal(out[schedule].normal_linear, out["wavefront"].normal_linear)
    _, _, alb, nrm = _oracle(scene, cam, aovs=True)
    a32, n32 = out["auto"].albedo_linear, out["auto"].normal_linear
    da = np.abs(a32 - alb).max(axis=2)
    dn = np.abs(n32 - nrm).max(axis=2)
    off = (da > 1e-5) | (dn > 1e-4)
    print(f"f32 AOVs: {int(off.sum())} of {off.size} pixels off by more than f32 rounding; "
          f"median |d albedo| {np.median(da):.2e}, median |d normal| {np.median(dn):.2e}")
    assert np.median(dn) <= 1e-6 and np.median(da) <= 1e-7
    assert off.mean() <= 0.01
    assert (alb.max(axis=2) > 0).mean() > 0.5


@pytest.mark.parametrize("mode", ["lambertian", "prefer_dielectric", "prefer_metal", "custom"])
def test_render_scene_material_modes_match_oracle(gpu_context, mode):
    ss = SurfaceScene()
    ground = np.array([[[-4, -1, 0], [4, -1, 0], [4, -1, -8]], [[-4, -1, 0], [4, -1, -8], [-4, -1, -8]]], float)
    ss.add_mesh(ground, material=SurfaceMaterial(base_color=(0.6, 0.6, 0.5), specular_color=(0.9, 0.9, 0.9)))
    cone = []
    for k in range(8):  # an eight-sided cone of triangles
        a0, a1 = 2 * np.pi * k / 8, 2 * np.pi * (k + 1) / 8
        cone.append([[0.0, 1.2, -4.0], [np.cos(a0), -1.0, -4.0 + np.sin(a0)], [np.cos(a1), -1.0, -4.0 + np.sin(a1)]])
    ss.add_mesh(np.array(cone), material=SurfaceMaterial(base_color=(0.2, 0.5, 0.8), specular_color=(0.8, 0.6, 0.4),
                                                         refractive_index=1.45))
    modes = {"lambertian": SurfaceRayMaterialMode.lambertian(),
             "prefer_dielectric": SurfaceRayMaterialMode.prefer_dielectric(),
             "prefer_metal": SurfaceRayMaterialMode.prefer_metal(0.2),
             "custom": SurfaceRayMaterialMode.custom(lambda m: RayMaterial.ggx_microfacet(m.specular_color, 0.35))}
    scene = ss.to_ray_scene_with_material_mode(modes[mode])
    cam = RayCamera(32, 1.0).with_samples_per_pixel(4).with_look_at((0, 0.5, 2), (0, 0, -4)).with_max_depth(8)
    img = PathTracer(cam, precision="f64", context=gpu_context).render_hdr_image(scene, want64=True)
    ref, acc = _oracle(scene, cam)
    assert rel_err(img.pixels64, ref, floor=1e-12).max() <= 1e-9
    np.testing.assert_array_equal(img.accepted, acc)
    img32 = PathTracer(cam, context=gpu_context).render_hdr_image(scene)
    ref32, _ = _oracle(scene, cam, precision=0)
    assert_explained(f"render_scene {mode}", scene, cam, img32.pixels, ref, ref32)
    if mode == "lambertian":  # render_scene_hdr_image compiles with the Lambertian policy
        direct = PathTracer(cam, precision="f64", context=gpu_context).render_scene_hdr_image(ss, want64=True)
        np.testing.assert_array_equal(direct.pixels64, img.pixels64)


def test_tone_mapped_render(gpu_context):
    # raytracing.rs:1504-1523: an empty world with background (4, 1, 0.25).
    tracer = PathTracer(RayCamera(1, 1.0).with_background((4.0, 1.0, 0.25)).with_samples_per_pixel(1),
                        context=gpu_context)
    world = RayScene()
    assert tuple(tracer.render(world)[0, 0]) == (255, 255, 128)
    tm = ToneMap().with_operator(TONE_MAP_REINHARD).with_gamma(1.0)
    assert tuple(tracer.render_tone_mapped(world, tm)[0, 0]) == (204, 128, 51)


def test_two_leaf_traversal_stats_on_the_gpu(gpu_context):
    # bvh.rs:666-709 through the device's f64 statistics walk.
    ids, t, st = two_leaf_scene().hit_rays(np.array([[0, 0, 0, 0, 0, 1, 0.0]]), t_min=0.0, t_max=20.0, ctx=gpu_context)
    assert ids[0] == 0 and t[0] == 1.0
    assert (st["rays"], st["node_bounds_tests"], st["node_bounds_hits"], st["leaf_visits"],
            st["primitive_candidates"], st["leaf_hit_results"]) == (1, 3, 3, 1, 1, 1)
