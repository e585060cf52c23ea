"""GPU parity: the CUDA path through the C ABI against the CPU oracle on the same inputs.

Checks (from the spec contract):
  1. primary-ray closest-hit primitive ids and BvhTraversalStats: bit-exact (f64 kernel);
  2. per-pixel radiance under identical RNG streams: the f64 wavefront matches the oracle
     to round-off; the f32 wavefront is within 1e-4 relative except on pixels where an f32
     rounding flipped a discrete decision (counted, bounded);
  3. converged images: relMSE of the f32 render against an f64 oracle render.
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from gartus_gb300 import abi, scenes
from gartus_gb300._lib import GartusError, check, lib
from gartus_gb300.raytracing import (EnvironmentLight, ImageTexture, PathTracer, RayCamera, RayGeometry, RayMaterial,
                                     RayScene, SamplingTargetList)
from tests.divergence import assert_explained, assert_modes_agree
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

# "wavefront": per-bounce kernels to the end; "auto": the wavefront hands its last slots
# to the persistent kernel (the default); "persistent": one persistent launch.
SCHEDULES = ["wavefront", "auto", "persistent"]


def relmse(x, r):
    return float(np.mean((x - r) ** 2 / (r * r + 1e-2)))


def probe_rays(seed):
    rr = scenes.SampleRng(seed ^ 0x9E3779B97F4A7C15)  # graphics/raytracing.rs:1344-1358
    rays = np.zeros((64, 7))
    for i in range(64):
        o = (rr.random_range(-4.0, 4.0), rr.random_range(-3.0, 3.0), rr.random_range(0.0, 3.0))
        t = (rr.random_range(-3.0, 3.0), rr.random_range(-2.0, 2.0), rr.random_range(-8.0, -1.0))
        rays[i, :3] = o
        rays[i, 3:6] = (t[0] - o[0], t[1] - o[1], t[2] - o[2])
    return rays


# -------------------------------------------------------------- check 1: hits
@pytest.mark.parametrize("name", ["final", "cornell", "bench"])
def test_primary_hits_and_stats_bit_exact(gpu_context, name):
    if name == "final":
        scene, cam, stride = scenes.final_scene_ray_scene(), scenes.final_scene_camera(160, 1), 1
    elif name == "cornell":
        scene, cam, stride = scenes.cornell_scene()[0], scenes.cornell_camera(96, 1), 1
    else:  # the reference bench's probe set: every 4th pixel (benches/render_performance.rs:42-50)
        scene, cam, stride = scenes.render_performance_scene(), scenes.render_performance_camera(), 4
    pt = PathTracer(cam, context=gpu_context)
    ids, t, stats = pt.trace_primary(scene, stride)
    o_ids, o_t, o_stats = oracle.OracleScene.from_ray_scene(scene).trace_primary(cam.desc(), stride)
    np.testing.assert_array_equal(ids, o_ids)
    np.testing.assert_array_equal(t, o_t)
    assert stats == o_stats
    assert scene.bvh_node_count(gpu_context) == oracle.OracleScene.from_ray_scene(scene).node_count()


def test_mesh_heavy_primary_hits_bit_exact(gpu_context):
    # The full 2,355,202-triangle mesh scene (Perlin height field + 64 tori): ids, hit
    # distances and traversal statistics of every 16th pixel's primary ray equal the
    # oracle's on the reference-layout BVH.
    scene, _ = scenes.mesh_heavy_scene(env_width=8, env_height=4)
    assert len(scene) == 2 * 1023 * 1023 + 64 * 4096
    cam = scenes.mesh_heavy_camera(1920, 1080, 1, 8)
    pt = PathTracer(cam, context=gpu_context)
    ids, t, stats = pt.trace_primary(scene, 16)
    o = oracle.OracleScene.from_ray_scene(scene)
    o_ids, o_t, o_stats = o.trace_primary(cam.desc(), 16)
    np.testing.assert_array_equal(ids, o_ids)
    np.testing.assert_array_equal(t, o_t)
    assert stats == o_stats
    assert (ids >= 0).mean() > 0.5  # the camera sees the height field
    assert scene.bvh_node_count(gpu_context) == o.node_count()


def test_randomized_scenes_match_oracle_and_bruteforce(gpu_context):
    # graphics/raytracing.rs:1340-1370 on the GPU: BVH hits equal brute force, stats equal.
    for seed in range(1, 17):
        scene = scenes.randomized_ray_scene(seed)
        rays = probe_rays(seed)
        ids, t, stats = scene.hit_rays(rays, ctx=gpu_context)
        o = oracle.OracleScene.from_ray_scene(scene)
        o_ids, o_t, _, o_stats = o.trace(rays)
        b_ids, b_t, _, _ = o.trace(rays, bruteforce=True)
        np.testing.assert_array_equal(ids, o_ids)
        np.testing.assert_array_equal(t, o_t)
        np.testing.assert_array_equal(ids >= 0, b_ids >= 0)
        assert stats == o_stats


def test_empty_scene_trace_and_render(gpu_context):
    scene = RayScene()
    scene.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    ids, _, stats = scene.hit_rays(np.array([[0, 0, 0, 0, 0, -1, 0.0]]), ctx=gpu_context)
    assert ids[0] == -1 and stats["rays"] == 1 and stats["node_bounds_tests"] == 0
    cam = RayCamera(3, 1.0).with_background((4.0, 2.0, 0.25)).with_samples_per_pixel(2)
    img = PathTracer(cam, context=gpu_context).render_hdr_image(scene)
    assert (img.pixels == np.array([4.0, 2.0, 0.25], dtype=np.float32)).all()
    assert (img.accepted == 2).all()


# ------------------------------------------------------ check 2: same streams
def _oracle_render(scene, cam, lights=None, env=None, precision=1, aovs=False):
    o = oracle.OracleScene.from_ray_scene(scene)
    la = lights.to_array() if lights is not None else None
    return o.render(cam.desc(), la, env, precision=precision, threads=8, aovs=aovs)


def _cases():
    final = scenes.final_scene_ray_scene()
    cornell, lights = scenes.cornell_scene()
    bench = scenes.render_performance_scene()
    return {
        "final": (final, scenes.final_scene_camera(64, 4), None),
        "cornell_mixture": (cornell, scenes.cornell_camera(40, 3, 50), lights),
        "cornell_nee": (cornell, scenes.cornell_camera(32, 2, 50).with_direct_lighting_mode(
            abi.GT_DIRECT_NEXT_EVENT_ESTIMATION), lights),
        "bench": (bench, scenes.render_performance_camera(), None),
    }


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("case", ["final", "cornell_mixture", "cornell_nee", "bench"])
def test_f64_path_matches_oracle(gpu_context, case, schedule):
    scene, cam, lights = _cases()[case]
    pt = PathTracer(cam, precision="f64", context=gpu_context, schedule=schedule)
    img = pt.render_with_lights_hdr_image(scene, lights, want64=True) if lights else pt.render_hdr_image(
        scene, want64=True)
    ref, acc = _oracle_render(scene, cam, lights)
    np.testing.assert_array_equal(img.accepted, acc)
    err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
    # The f64 kernels repeat the reference's arithmetic operation for operation; only
    # CUDA's sin/cos/acos/atan2 may differ from glibc in the last ulp, so every pixel
    # agrees far inside the 1e-4 bound (observed: <= 1e-12 relative).
    print(f"{case}: f64 max relative error {err.max():.3e}")
    assert err.max() <= 1e-9



@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("case", ["final", "cornell_mixture", "cornell_nee", "bench"])
def test_f32_path_same_streams(gpu_context, case, schedule):
    # Same RNG streams in f32.  A pixel may leave the f64 reference by more than 1e-4 only
    # where f32 rounding flipped one of its samples' decisions (a hit at an edge or
    # silhouette, a Schlick or total-internal-reflection choice, Russian roulette, ...) or
    # where the f32 restatement of the reference drifts as well (tests/divergence.py);
    # every such pixel is counted by cause, with no slack.
    scene, cam, lights = _cases()[case]
    pt = PathTracer(cam, precision="f32", context=gpu_context, schedule=schedule)
    img = pt.render_with_lights_hdr_image(scene, lights) if lights else pt.render_hdr_image(scene)
    ref64, acc = _oracle_render(scene, cam, lights)
    ref32, _ = _oracle_render(scene, cam, lights, precision=0)
    assert_explained(f"{case}/{schedule}", scene, cam, img.pixels, ref64, ref32, lights)
    np.testing.assert_array_equal(img.accepted, acc)
    err = rel_err(img.pixels, ref64, floor=1e-3).max(axis=2)
    assert float(np.median(err)) <= 1e-5
    assert np.isfinite(img.pixels).all()


def test_converged_relmse_against_f64_oracle(gpu_context):
    # Check 3 at 576 spp.  (a) Independent streams: the f32 GPU image's relMSE against an
    # f64 oracle image is no larger than the noise floor between two f64 oracle images,
    # i.e. f32 adds no bias.  (b) Same streams, so sampling noise cancels: pixels whose
    # 576 samples took the same decisions agree to relMSE 1e-8; the few with a flipped
    # decision (a caustic sample through the glass sphere can dominate a pixel) are
    # counted: the implied per-sample flip rate stays under 5e-4.
    scene, lights = scenes.cornell_scene()
    cam = scenes.cornell_camera(24, 24, 50)
    img = PathTracer(cam, context=gpu_context).render_with_lights_hdr_image(scene, lights)
    x = img.pixels.astype(np.float64)
    same, _ = _oracle_render(scene, cam, lights)
    other, _ = _oracle_render(scene, cam.with_rng_seed(12345), lights)
    e_gpu = relmse(x, other)
    e_floor = relmse(same, other)
    err = rel_err(x, same, floor=1e-3).max(axis=2)
    keep = err <= 1e-4
    e_same_kept = relmse(x[keep], same[keep])
    print(f"relMSE independent streams: gpu-f32 {e_gpu:.3e} vs f64 noise floor {e_floor:.3e}; "
          f"same streams: {int((~keep).sum())} pixels with a flipped sample of {keep.size}, "
          f"relMSE of the rest {e_same_kept:.3e}")
    assert e_gpu <= 1.1 * e_floor + 1e-4
    # Per-sample flip rate: a pixel stays clean only if all of its spp samples do.
    spp = 24 * 24
    rate = -math.log(max(1.0 - float((~keep).mean()), 1e-12)) / spp
    assert rate <= 5e-4
    assert e_same_kept <= 1e-8


def test_aovs_match_oracle(gpu_context):
    # render_denoising_aovs (camera.rs:4187-4244): albedo and normal AOVs.
    scene = scenes.final_scene_ray_scene()
    cam = scenes.final_scene_camera(48, 3)
    aovs = PathTracer(cam, precision="f64", context=gpu_context).render_denoising_aovs(scene)
    _, _, alb, nrm = _oracle_render(scene, cam, aovs=True)
    np.testing.assert_allclose(aovs.albedo_linear, alb, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(aovs.normal_linear, nrm, rtol=1e-6, atol=1e-6)


def _env_u8(seed=3, w=16, h=8):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 256, size=(h, w, 3), dtype=np.uint8)


@pytest.mark.parametrize("fmt", ["srgb8", "rgb32f"])
def test_environment_light_matches_oracle(gpu_context, fmt):
    # render_with_environment_hdr_image (renderer.rs:431-449): forced NEE, env MIS.
    texels = _env_u8()
    if fmt == "rgb32f":
        texels = (texels.astype(np.float32) / 255.0) ** 2 * 4.0
    env = EnvironmentLight(texels)
    scene = scenes.render_performance_scene()
    cam = scenes.render_performance_camera().with_samples_per_pixel(3)
    img = PathTracer(cam, precision="f64", context=gpu_context).render_with_environment_hdr_image(
        scene, env, want64=True)
    ref, acc = _oracle_render(scene, cam, env=env)
    err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
    assert (err <= 1e-9).mean() >= 0.99
    assert (err <= 1e-4).mean() >= 0.995
    img32 = PathTracer(cam, precision="f32", context=gpu_context).render_with_environment_hdr_image(scene, env)
    ref32, _ = _oracle_render(scene, cam, env=env, precision=0)
    assert_explained(f"environment {fmt}", scene, cam, img32.pixels, ref, ref32, env=env)


def test_adaptive_sampling_matches_oracle(gpu_context):
    # render_world_pixel_adaptive (camera.rs:2937-2982): Welford stopping rule.
    scene = scenes.final_scene_ray_scene()
    # The threshold avoids 0.05, which sky pixels whose samples are exactly 1.0 and 0.5
    # reach exactly in real arithmetic (a tie decided by the last ulp of sin/cos).
    cam = scenes.final_scene_camera(40, 1).with_adaptive_sampling(4, 24, 0.0473)
    img = PathTracer(cam, precision="f64", context=gpu_context).render_hdr_image(scene, want64=True)
    ref, acc = _oracle_render(scene, cam)
    assert (img.accepted != acc).sum() <= 0.005 * acc.size
    err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
    assert (err <= 1e-9).mean() >= 0.99


def test_moving_spheres_and_checker(gpu_context):
    scene = RayScene()
    chk = scene.add_material(RayMaterial.checker_lambertian(0.5, (0.9, 0.9, 0.9), (0.2, 0.3, 0.1)))
    scene.add_sphere((0.0, -100.5, -1.0), 100.0, chk)
    blur = scene.add_material(RayMaterial.lambertian((0.7, 0.3, 0.3)))
    scene.add_moving_sphere((0.0, 0.0, -1.0), (0.0, 0.3, -1.0), 0.5, blur)
    iso = scene.add_material(RayMaterial.isotropic((0.5, 0.6, 0.7)))
    scene.add_sphere((1.1, 0.0, -1.2), 0.3, iso)
    scene.build_bvh()
    cam = RayCamera(48, 1.5).with_samples_per_pixel(4).with_max_depth(8)
    img = PathTracer(cam, precision="f64", context=gpu_context).render_hdr_image(scene, want64=True)
    ref, _ = _oracle_render(scene, cam)
    err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
    assert (err <= 1e-9).mean() >= 0.99


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_mesh_heavy_small(gpu_context, precision):
    # The mesh-heavy generator at a small size: triangle meshes, GGX everywhere, an f32
    # HDR sky with a 5e4 sun (next-event estimation forced by the environment).
    scene, env = scenes.mesh_heavy_scene(size=40, tori=6, rings=8, tube=12, env_width=256, env_height=128)
    cam = scenes.mesh_heavy_camera(48, 27, 2, 8)
    pt = PathTracer(cam, precision=precision, context=gpu_context)
    ref, acc = _oracle_render(scene, cam, env=env)
    if precision == "f64":
        img = pt.render_with_environment_hdr_image(scene, env, want64=True)
        np.testing.assert_array_equal(img.accepted, acc)
        err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
        assert (err <= 1e-9).mean() >= 0.99, err.max()
    else:
        img = pt.render_with_environment_hdr_image(scene, env)
        ref32, _ = _oracle_render(scene, cam, env=env, precision=0)
        assert_explained("mesh-heavy small", scene, cam, img.pixels, ref, ref32, env=env)
    assert np.isfinite(img.pixels).all()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_noise_textures(gpu_context, precision):
    # NoiseTexture plain, turbulence and marble (graphics/raytracing/texture.rs:278-352)
    # on Lambertian spheres; the Perlin tables are made on the host in f64.
    scene = RayScene()
    ground = scene.add_material(RayMaterial.noise_lambertian(4.0, seed=7))
    scene.add_sphere((0.0, -1000.0, 0.0), 1000.0, ground)
    marble = scene.add_material(RayMaterial.marble_lambertian(4.0, seed=3))
    scene.add_sphere((0.0, 2.0, 0.0), 2.0, marble)
    turb = scene.add_material(RayMaterial.turbulence_lambertian(2.5, depth=5, seed=11))
    scene.add_sphere((3.5, 1.0, 1.5), 1.0, turb)
    scene.build_bvh()
    cam = (RayCamera(48, 1.5).with_samples_per_pixel(4).with_max_depth(6).with_vertical_fov(20.0)
           .with_look_at((13.0, 2.0, 3.0), (0.0, 2.0, 0.0)))
    pt = PathTracer(cam, precision=precision, context=gpu_context)
    ref, acc = _oracle_render(scene, cam)
    if precision == "f64":
        img = pt.render_hdr_image(scene, want64=True)
        np.testing.assert_array_equal(img.accepted, acc)
        err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
        assert err.max() <= 1e-9, err.max()
    else:
        img = pt.render_hdr_image(scene)
        ref32, _ = _oracle_render(scene, cam, precision=0)
        assert_explained("noise textures", scene, cam, img.pixels, ref, ref32)
        assert np.median(rel_err(img.pixels, ref, floor=1e-3)) <= 1e-5
    # the textures vary over the image: not a constant grey
    assert np.std(ref) > 1e-3


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_batch_matches_single_frames(gpu_context, precision):
    # gt_render_batch: frames with different poses, seeds, adaptive minimums and sizes in
    # one launch give each frame's gt_render image (bit-identical in f64).
    scene, lights = scenes.batch_scene()
    cams = scenes.batch_cameras(frames=5, width=20, spp_cycle=(2, 4, 8), max_samples=16, threshold=0.05)
    cams.append(scenes.cornell_camera(12, 2, 20))  # a stratified frame of another size
    pt = PathTracer(cams[0], precision=precision, context=gpu_context)
    imgs = pt.render_batch_hdr_images(scene, cams, lights=lights, want64=precision == "f64")
    assert pt.last_stats["samples"] == sum(int(i.accepted.sum()) for i in imgs)
    for cam, img in zip(cams, imgs):
        one = PathTracer(cam, precision=precision, context=gpu_context).render_with_lights_hdr_image(
            scene, lights, want64=precision == "f64")
        np.testing.assert_array_equal(img.accepted, one.accepted)
        if precision == "f64":
            np.testing.assert_array_equal(img.pixels64, one.pixels64)
        else:
            assert_modes_agree("batch frame vs single frame", scene, cam, img.pixels, one.pixels, lights)
    if precision == "f64":  # and the oracle agrees on one frame
        ref, acc = _oracle_render(scene, cams[1], lights)
        np.testing.assert_array_equal(imgs[1].accepted, acc)
        assert rel_err(imgs[1].pixels64, ref, floor=1e-12).max() <= 1e-9


@pytest.mark.parametrize("schedule", ["auto", "wavefront"])
def test_batch_wavefront_matches_single_frames(gpu_context, schedule):
    # Frames of one width in f32 run through the striped wavefront as one image of their
    # rows: every frame equals its own gt_render (the same accepted counts; radiance within
    # the f32 tolerance, as the batch kernels are separate instantiations).  Eight frames
    # of 48x48 with adaptive sampling exercise the stripes, the migration and the tail.
    scene, lights = scenes.batch_scene()
    cams = scenes.batch_cameras(frames=8, width=48, spp_cycle=(4, 8, 16), max_samples=64, threshold=0.05)
    cams.append(scenes.cornell_camera(48, 3, 20))  # a stratified frame of the same width
    pt = PathTracer(cams[0], context=gpu_context, schedule=schedule)
    imgs = pt.render_batch_hdr_images(scene, cams, lights=lights)
    assert pt.last_stats["samples"] == sum(int(i.accepted.sum()) for i in imgs)
    assert pt.last_stats["iterations"] > 1  # the wavefront ran (the persistent batch reports 1)
    for cam, img in zip(cams, imgs):
        one = PathTracer(cam, context=gpu_context).render_with_lights_hdr_image(scene, lights)
        flipped = int((img.accepted != one.accepted).sum())
        assert flipped <= 0.02 * img.accepted.size, flipped
        assert_modes_agree("striped batch frame vs single frame", scene, cam, img.pixels, one.pixels, lights)


def test_autotune_keeps_the_image(gpu_context):
    # gt_autotune times candidate stripe counts, tail sizes and blocks per SM on the frame
    # and keeps the fastest; launch shapes never change the image.
    scene, lights = scenes.cornell_scene()
    cam = scenes.cornell_camera(64, 4, 20)
    base = PathTracer(cam, context=gpu_context).render_with_lights_hdr_image(scene, lights)
    pt = PathTracer(cam, context=gpu_context)
    rep = pt.autotune(scene, lights)
    print("autotune:", rep)
    assert rep["trials"] >= 10
    assert rep["best_ms"] <= rep["given_ms"]
    assert 0 <= rep["stripes"] <= 8 and 0 <= rep["trace_blocks_per_sm"] <= 32
    assert rep["schedule"] in ("auto", "persistent") and pt.schedule == rep["schedule"]
    tuned = pt.render_with_lights_hdr_image(scene, lights)
    np.testing.assert_array_equal(tuned.accepted, base.accepted)
    if rep["schedule"] == "auto" and rep["migrate"] == "default":
        np.testing.assert_array_equal(tuned.pixels, base.pixels)
    else:  # other kernels finish (some) pixels, fusing f32 operations differently
        assert_modes_agree("autotuned vs default", scene, cam, tuned.pixels, base.pixels, lights)
    # a batch tunes the same way
    cams = scenes.batch_cameras(frames=3, width=32, spp_cycle=(4,), max_samples=8)
    rep = PathTracer(cams[0], context=gpu_context).autotune(scene, lights, cameras=cams)
    assert rep["trials"] >= 10
    # tuning the same tracer again (after a tune that may have chosen the persistent
    # schedule) tunes from AUTO
    again = pt.autotune(scene, lights)
    assert again["trials"] >= 10 and again["schedule"] in ("auto", "persistent")
    assert PathTracer(cam, context=gpu_context, schedule="persistent").autotune(scene, lights)["trials"] >= 10


def test_batch_rejects_bad_jobs(gpu_context):
    scene, lights = scenes.batch_scene()
    cam = scenes.batch_cameras(frames=1, width=8)[0]
    with pytest.raises(GartusError) as e:
        PathTracer(cam, context=gpu_context).render_batch_hdr_images(scene, [], lights=lights)
    assert e.value.status == abi.GT_ERR_INVALID_ARG
    f = abi.gt_frame()
    f.struct_size = C.sizeof(abi.gt_frame)
    buf = np.zeros((4, 4, 3), dtype=np.float32)
    f.width, f.height, f.rgb = 4, 4, buf.ctypes.data  # 8x8 camera, 4x4 frame
    jobs = (abi.gt_frame_job * 1)()
    d = cam.desc()
    jobs[0].camera = C.pointer(d)
    jobs[0].frame = C.pointer(f)
    o = abi.gt_render_opts()
    o.struct_size = C.sizeof(abi.gt_render_opts)
    assert lib().gt_render_batch(scene._handle(gpu_context).h, None, None, jobs, 1, C.byref(o)) == abi.GT_ERR_INVALID_ARG
    f.width, f.height = 8, 8
    buf8 = np.zeros((8, 8, 3), dtype=np.float32)
    f.rgb = buf8.ctypes.data
    o.aovs = 1
    assert lib().gt_render_batch(scene._handle(gpu_context).h, None, None, jobs, 1, C.byref(o)) == abi.GT_ERR_UNSUPPORTED
    o.aovs = 0
    assert lib().gt_render_batch(scene._handle(gpu_context).h, None, None, jobs, 1, C.byref(o)) == abi.GT_OK
    assert np.isfinite(buf8).all() and buf8.max() > 0


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_accumulate_equals_one_render(gpu_context, precision):
    # gt_render_accumulate: 3 + 5 + 8 samples on one accumulator (with a host checkpoint
    # and restore in between) give the image of one 16-sample render: each pixel's stream
    # and Kahan sums simply continue.
    from gartus_gb300.raytracing import Accumulator
    scene, lights = scenes.cornell_scene()
    base = scenes.cornell_camera(40, 1, 50).with_pixel_sample_mode(abi.GT_SAMPLE_RANDOM)
    full = PathTracer(base.with_samples_per_pixel(16), precision=precision,
                      context=gpu_context).render_with_lights_hdr_image(scene, lights, want64=precision == "f64")
    pt = PathTracer(base, context=gpu_context)
    acc = Accumulator(40, 40, precision, gpu_context)
    pt.render_accumulate(scene, acc, 3, lights=lights)
    blob = acc.save()
    acc2 = Accumulator(40, 40, precision, gpu_context)
    acc2.load(blob)
    assert acc2.samples == 3
    pt.render_accumulate(scene, acc2, 5, lights=lights)
    img = pt.render_accumulate(scene, acc2, 8, lights=lights)
    assert acc2.samples == 16
    np.testing.assert_array_equal(img.accepted, full.accepted)
    if precision == "f64":
        np.testing.assert_array_equal(img.pixels64, full.pixels64)
    else:  # the chunks may finish pixels in other kernels, which fuse f32 operations differently
        assert_modes_agree("accumulated vs one render", scene, base.with_samples_per_pixel(16), img.pixels,
                           full.pixels, lights)
    # Misuse is rejected: a stratified camera, another seed, a size mismatch.
    with pytest.raises(GartusError) as e:
        PathTracer(scenes.cornell_camera(40, 2, 50), context=gpu_context).render_accumulate(scene, acc2, 1, lights=lights)
    assert e.value.status == abi.GT_ERR_UNSUPPORTED
    with pytest.raises(GartusError):
        PathTracer(base.with_rng_seed(99), context=gpu_context).render_accumulate(scene, acc2, 1, lights=lights)
    with pytest.raises(GartusError):
        Accumulator(8, 8, precision, gpu_context).load(blob)


def test_edge_cases(gpu_context):
    scene = scenes.final_scene_ray_scene()
    # max_depth 0: the bounce loop never runs, every sample is black (camera.rs:1742).
    img = PathTracer(scenes.final_scene_camera(8, 2).with_max_depth(0), context=gpu_context).render_hdr_image(scene)
    assert (img.pixels == 0).all() and (img.accepted == 2).all()
    # A 1x1 image.
    img = PathTracer(RayCamera(1, 1.0).with_samples_per_pixel(3), context=gpu_context).render_hdr_image(scene)
    assert img.pixels.shape == (1, 1, 3) and np.isfinite(img.pixels).all()
    # Russian roulette off, deep paths.
    cam = scenes.final_scene_camera(16, 2).without_russian_roulette().with_max_depth(30)
    img = PathTracer(cam, precision="f64", context=gpu_context).render_hdr_image(scene, want64=True)
    ref, _ = _oracle_render(scene, cam)
    assert (rel_err(img.pixels64, ref, floor=1e-12).max(axis=2) <= 1e-9).mean() >= 0.99


def test_invalid_arguments_return_status(gpu_context):
    from gartus_gb300.raytracing import _SceneHandle, PRIMITIVE_DTYPE, MATERIAL_DTYPE
    prims = np.zeros(1, dtype=PRIMITIVE_DTYPE)
    prims[0]["geometry"]["kind"] = abi.GT_GEOM_SPHERE
    prims[0]["geometry"]["p"][3] = 1.0
    prims[0]["material"] = 3  # out of bounds (scene.rs:1158-1161 panics)
    mats = np.zeros(1, dtype=MATERIAL_DTYPE)
    with pytest.raises(GartusError) as e:
        _SceneHandle(gpu_context, prims, mats, 4)
    assert e.value.status == abi.GT_ERR_INVALID_ARG
    # A frame whose size does not match the camera.
    scene = scenes.final_scene_ray_scene()
    cam = RayCamera(8, 1.0)
    f = abi.gt_frame()
    f.struct_size = C.sizeof(abi.gt_frame)
    buf = np.zeros((9, 8, 3), dtype=np.float32)
    f.width, f.height, f.rgb = 8, 9, buf.ctypes.data
    st = lib().gt_render(scene._handle(gpu_context).h, None, None, C.byref(cam.desc()), None, C.byref(f))
    assert st == abi.GT_ERR_INVALID_ARG
    # Non-positive light weight (scene.rs:460-465).
    lights = SamplingTargetList()
    with pytest.raises(ValueError):
        lights.add_target_weighted(RayGeometry.sphere((0, 0, 0), 1), 0.0)


def test_progress_callback_can_cancel(gpu_context):
    scene, lights = scenes.cornell_scene()
    cam = scenes.cornell_camera(64, 8, 50)
    calls = []

    @abi.GT_PROGRESS_FN
    def cb(user, done, total):
        calls.append((done, total))
        return 1  # cancel at the first report

    f = abi.gt_frame()
    f.struct_size = C.sizeof(abi.gt_frame)
    buf = np.zeros((64, 64, 3), dtype=np.float32)
    f.width, f.height, f.rgb = 64, 64, buf.ctypes.data
    o = abi.gt_render_opts()
    o.struct_size = C.sizeof(abi.gt_render_opts)
    o.progress = cb
    o.schedule = abi.GT_SCHEDULE_WAVEFRONT
    st = lib().gt_render(scene._handle(gpu_context).h, lights._handle(gpu_context).h, None, C.byref(cam.desc()),
                         C.byref(o), C.byref(f))
    assert st == abi.GT_ERR_CANCELLED and len(calls) == 1
    # The context stays usable after a cancelled render.
    img = PathTracer(scenes.cornell_camera(16, 1, 5), context=gpu_context).render_with_lights_hdr_image(scene, lights)
    assert np.isfinite(img.pixels).all()


@pytest.mark.parametrize("schedule", ["auto", "persistent"])
def test_render_progressive(gpu_context, schedule):
    # PathTracer::render_progressive (renderer.rs:136-146): updates carry the image as far
    # as it is known; finished pixels already hold their final values.
    scene, lights = scenes.cornell_scene()
    cam = scenes.cornell_camera(320, 4, 50)
    pt = PathTracer(cam, context=gpu_context, schedule=schedule)
    seen = []
    img = pt.render_progressive(scene, lambda u: seen.append((u.completed, u.total, u.pixels.copy())), lights=lights)
    # The same image as a plain render: f32 renders are reproducible, because every slot's
    # kernel is chosen by deterministic rules and both persistent modes share one code.
    final = pt.render_with_lights_hdr_image(scene, lights)
    np.testing.assert_array_equal(img.pixels, final.pixels)
    assert seen and all(0 <= c <= t for c, t, _ in seen)
    for _, _, px in seen:  # every channel is 0 (not yet known) or final
        assert ((px == 0) | (px == img.pixels)).all()

    class Stop(Exception):
        pass

    def stop(u):
        raise Stop()

    with pytest.raises(Stop):
        pt.render_progressive(scene, stop, lights=lights)
    assert np.isfinite(pt.render_with_lights_hdr_image(scene, lights).pixels).all()


@pytest.mark.parametrize("schedule", ["wavefront", "persistent"])
def test_calls_from_inside_a_progress_callback(gpu_context, schedule):
    # The progress callback runs on the rendering thread while the render holds the
    # context.  A handle released there (the last reference dropped, as when the garbage
    # collector finalises it) is destroyed once the render returns; any other call on the
    # context fails with GT_ERR_INVALID_ARG instead of deadlocking.
    scene, lights = scenes.cornell_scene()
    doomed = [scenes.cornell_scene()[0]]
    doomed[0]._handle(gpu_context)  # resident on the device
    pt = PathTracer(scenes.cornell_camera(256, 4, 50), context=gpu_context, schedule=schedule)
    errors = []

    def progress(update):
        if doomed:
            doomed.pop()  # gt_scene_destroy from inside the callback
            try:
                PathTracer(scenes.cornell_camera(16, 1, 5), context=gpu_context).render_with_lights_hdr_image(
                    scene, lights)
            except GartusError as e:
                errors.append(str(e))

    img = pt.render_progressive(scene, progress, lights=lights)
    assert not doomed and np.isfinite(img.pixels).all()
    assert len(errors) == 1 and "progress callback" in errors[0], errors
    again = pt.render_with_lights_hdr_image(scene, lights)
    np.testing.assert_array_equal(again.pixels, img.pixels)


def test_persistent_progress_and_cancel(gpu_context):
    # The persistent kernel polls a host-mapped cancel word between pixels; the host
    # reports progress while it runs.  A cancelled render returns GT_ERR_CANCELLED and
    # leaves the context usable.
    scene, lights = scenes.cornell_scene()
    cam = scenes.cornell_camera(512, 16, 50)
    seen = []

    @abi.GT_PROGRESS_FN
    def cb(user, done, total):
        seen.append((done, total))
        return 1 if len(seen) >= 2 else 0

    w, h, _ = cam.image_size()
    buf = np.zeros((h, w, 3), dtype=np.float32)
    f = abi.gt_frame()
    f.struct_size = C.sizeof(abi.gt_frame)
    f.width, f.height, f.rgb = w, h, buf.ctypes.data
    o = abi.gt_render_opts()
    o.struct_size = C.sizeof(abi.gt_render_opts)
    o.progress = cb
    o.schedule = abi.GT_SCHEDULE_PERSISTENT
    st = lib().gt_render(scene._handle(gpu_context).h, lights._handle(gpu_context).h, None, C.byref(cam.desc()),
                         C.byref(o), C.byref(f))
    assert st in (abi.GT_OK, abi.GT_ERR_CANCELLED)
    assert all(d <= t for d, t in seen)
    img = PathTracer(scenes.cornell_camera(16, 1, 5), context=gpu_context,
                     schedule="persistent").render_with_lights_hdr_image(scene, lights)
    assert np.isfinite(img.pixels).all()


@pytest.mark.parametrize("schedule,tail,grid,width,stripes", [("wavefront", 0, 4, 48, 0), ("auto", 100, 4, 48, 0),
                                                             ("auto", 1000000, 4, 48, 0), ("auto", 1, 8, 48, 0),
                                                             ("auto", 1000000, 4, 96, 0), ("wavefront", 0, 4, 50, 1),
                                                             ("wavefront", 0, 4, 50, 3), ("auto", 1, 8, 50, 8)])
def test_schedules_agree(gpu_context, schedule, tail, grid, width, stripes):
    # Every schedule evaluates the same per-pixel arithmetic in the same order: bit-identical
    # in f64 (no fused multiply-add anywhere), whether the wavefront runs to the end, hands
    # its last 100 slots to the persistent kernel, hands over at once, or (64 samples per
    # pixel, tail of one slot) first moves its slowest pixels to the concurrent persistent
    # kernel.  At 96x96 the tail starts one slot per lane and hands its last slots to one
    # warp each mid-path; 1, 3 (rows not a multiple) and 8 wavefront stripes.  In f32 the compiler may fuse differently in the kernels, so
    # images agree to f32 rounding.
    scene, lights = scenes.cornell_scene()
    cam = scenes.cornell_camera(width, grid, 50)
    a = PathTracer(cam, precision="f64", context=gpu_context, schedule=schedule, tail_slots=tail, stripes=stripes)
    b = PathTracer(cam, precision="f64", context=gpu_context, schedule="persistent")
    ia = a.render_with_lights_hdr_image(scene, lights, want64=True)
    ib = b.render_with_lights_hdr_image(scene, lights, want64=True)
    np.testing.assert_array_equal(ia.pixels64, ib.pixels64)
    np.testing.assert_array_equal(ia.accepted, ib.accepted)
    assert a.last_stats["samples"] == b.last_stats["samples"]
    assert a.last_stats["rays"] == b.last_stats["rays"]
    if grid == 8:
        assert a.last_stats["migrated_pixels"] > 0
    if schedule == "wavefront":
        assert a.last_stats["migrated_pixels"] == 0 and a.last_stats["tail_pixels"] == 0
    fa = PathTracer(cam, context=gpu_context, schedule=schedule, tail_slots=tail,
                    stripes=stripes).render_with_lights_hdr_image(scene, lights)
    fb = PathTracer(cam, context=gpu_context, schedule="persistent").render_with_lights_hdr_image(scene, lights)
    assert_modes_agree(f"{schedule} vs persistent", scene, cam, fa.pixels, fb.pixels, lights)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_henyey_greenstein_spheres(gpu_context, precision):
    # HenyeyGreenstein (material.rs:1175-1333): forward, backward and nearly isotropic
    # (|g| < 1e-3 takes the isotropic branch) phase functions around the incoming ray.
    scene = RayScene()
    ground = scene.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    scene.add_sphere((0.0, -100.5, -1.0), 100.0, ground)
    for x, g in ((-1.1, 0.6), (0.0, -0.4), (1.1, 0.0005)):
        scene.add_sphere((x, 0.0, -1.2), 0.5, scene.add_material(RayMaterial.henyey_greenstein((0.8, 0.7, 0.6), g)))
    scene.build_bvh()
    cam = RayCamera(48, 1.5).with_samples_per_pixel(8).with_max_depth(10)
    ref, acc = _oracle_render(scene, cam)
    if precision == "f64":
        img = PathTracer(cam, precision="f64", context=gpu_context).render_hdr_image(scene, want64=True)
        np.testing.assert_array_equal(img.accepted, acc)
        err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
        assert (err <= 1e-9).mean() >= 0.99, err.max()
    else:
        img = PathTracer(cam, context=gpu_context).render_hdr_image(scene)
        ref32, _ = _oracle_render(scene, cam, precision=0)
        assert_explained("henyey-greenstein", scene, cam, img.pixels, ref, ref32)
    with pytest.raises(ValueError):
        RayMaterial.henyey_greenstein((0.5, 0.5, 0.5), 1.0)


def test_gpu_bvh_matches_reference_tree(gpu_context):
    # GT_BVH_GPU_LBVH: the f32 path traverses a tree built on the device (Morton order,
    # Karras 2012).  The closest hits are the same primitives as with the reference SAH tree
    # (only exact ties may resolve differently), so the f32 images agree with the SAH
    # tree's and with the oracle within the f32 tolerance; f64 still uses the SAH tree.
    scene, env = scenes.mesh_heavy_scene(size=40, tori=6, rings=8, tube=12, env_width=256, env_height=128)
    cam = scenes.mesh_heavy_camera(48, 27, 2, 8)
    sah = PathTracer(cam, context=gpu_context).render_with_environment_hdr_image(scene, env)
    scene.use_gpu_bvh()
    gpu = PathTracer(cam, context=gpu_context).render_with_environment_hdr_image(scene, env)
    np.testing.assert_array_equal(gpu.accepted, sah.accepted)
    assert_modes_agree("linear BVH vs SAH tree", scene, cam, gpu.pixels, sah.pixels, env=env)
    ref, _ = _oracle_render(scene, cam, env=env)
    img64 = PathTracer(cam, precision="f64", context=gpu_context).render_with_environment_hdr_image(scene, env,
                                                                                                  want64=True)
    err = rel_err(img64.pixels64, ref, floor=1e-12).max(axis=2)
    assert (err <= 1e-9).mean() >= 0.99
    assert scene.bvh_node_count(gpu_context) > 0  # the reference tree, built on demand


def test_gpu_bvh_edge_cases(gpu_context):
    cam = RayCamera(16, 1.0).with_samples_per_pixel(2).with_max_depth(4).with_look_at((0, 0, 3), (0, 0, 0))
    # one primitive (a leaf root) and an empty scene
    for count in (1, 0):
        s = RayScene()
        m = s.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
        for _ in range(count):
            s.add_sphere((0.0, 0.0, 0.0), 0.5, m)
        s.build_bvh()
        a = PathTracer(cam, context=gpu_context).render_hdr_image(s)
        s.use_gpu_bvh()
        b = PathTracer(cam, context=gpu_context).render_hdr_image(s)
        np.testing.assert_array_equal(a.pixels, b.pixels)
    # many primitives with one box centre: equal Morton codes, split by index
    s = RayScene()
    m = s.add_material(RayMaterial.lambertian((0.5, 0.6, 0.7)))
    for k in range(300):
        r = 0.2 + 0.001 * k
        s.add_sphere((0.0, 0.0, 0.0), r, m)
    s.add_sphere((0.0, -100.5, 0.0), 100.0, m)
    s.build_bvh()
    a = PathTracer(cam, context=gpu_context).render_hdr_image(s)
    s.use_gpu_bvh()
    b = PathTracer(cam, context=gpu_context).render_hdr_image(s)
    assert_modes_agree("linear BVH, one box centre", s, cam, b.pixels, a.pixels)


def _textured_scene():
    rng = np.random.default_rng(77)
    checker = np.zeros((8, 8, 3), np.uint8)
    checker[(np.arange(8)[:, None] + np.arange(8)[None, :]) % 2 == 0] = (230, 200, 40)
    checker[(np.arange(8)[:, None] + np.arange(8)[None, :]) % 2 == 1] = (30, 60, 200)
    noise = rng.integers(0, 256, size=(13, 17, 3), dtype=np.uint8)
    floor_tex = ImageTexture(checker, filter="linear", wrap_s="repeat", wrap_t="repeat")
    ball_tex = ImageTexture(noise)  # nearest, clamped
    tri_tex = ImageTexture(noise[:5, :7], filter="linear")
    lamp_tex = ImageTexture(np.full((2, 2, 3), 255, np.uint8))
    scene = RayScene()
    scene.add_quad((-3.0, -0.5, -4.0), (6.0, 0.0, 0.0), (0.0, 0.0, 5.0),
                   scene.add_material(RayMaterial.textured_lambertian(floor_tex)))
    scene.add_sphere((-0.6, 0.1, -1.4), 0.55, scene.add_material(RayMaterial.textured_lambertian(ball_tex)))
    scene.add_sphere((0.7, 0.0, -1.1), 0.4, scene.add_material(RayMaterial.textured_ggx_microfacet(ball_tex, 0.4)))
    scene.add_triangle((0.2, -0.5, -2.2), (1.6, -0.5, -2.0), (0.9, 0.9, -2.4),
                       scene.add_material(RayMaterial.textured_lambertian(tri_tex)))
    scene.add_quad((-1.0, 2.0, -2.0), (2.0, 0.0, 0.0), (0.0, 0.0, 1.0),
                   scene.add_material(RayMaterial.textured_diffuse_light(lamp_tex)))
    scene.build_bvh()
    return scene


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_image_textures(gpu_context, precision):
    # ImageTexture (raytracing/texture.rs:110-156) on a quad (linear, repeated), spheres
    # (nearest, clamped; Lambertian and GGX) and a triangle, lit by a textured emitter;
    # (u, v) come from sphere_uv, the quad's plane coordinates and the barycentrics.
    scene = _textured_scene()
    assert len(scene.images()) == 4
    cam = (RayCamera(64, 1.5).with_samples_per_pixel(6).with_max_depth(8)
           .with_background((0.05, 0.05, 0.08)))
    ref, acc = _oracle_render(scene, cam)
    if precision == "f64":
        img = PathTracer(cam, precision="f64", context=gpu_context).render_hdr_image(scene, want64=True)
        np.testing.assert_array_equal(img.accepted, acc)
        err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
        assert (err <= 1e-9).mean() >= 0.99, err.max()
    else:
        img = PathTracer(cam, context=gpu_context).render_hdr_image(scene)
        ref32, _ = _oracle_render(scene, cam, precision=0)
        assert_explained("image textures", scene, cam, img.pixels, ref, ref32)
    assert np.std(ref) > 1e-3


def test_image_texture_edge_cases(gpu_context):
    # an empty bitmap samples cyan; a texture index past the image table is rejected
    scene = RayScene()
    scene.add_quad((-2.0, -2.0, -1.0), (4.0, 0.0, 0.0), (0.0, 4.0, 0.0),
                   scene.add_material(RayMaterial.textured_diffuse_light(ImageTexture(np.zeros((0, 0, 3), np.uint8)))))
    scene.build_bvh()
    cam = RayCamera(8, 1.0).with_samples_per_pixel(1).with_max_depth(2)
    img = PathTracer(cam, precision="f64", context=gpu_context).render_hdr_image(scene, want64=True)
    np.testing.assert_array_equal(img.pixels64[4, 4], [0.0, 1.0, 1.0])
    bad = scene.materials_array()
    bad[0]["tex"][0] = 1.0
    with pytest.raises(GartusError):
        from gartus_gb300.raytracing import _SceneHandle
        _SceneHandle(gpu_context, scene.primitives_array(), bad, 4, abi.GT_BVH_REFERENCE_SAH, scene.images())


def _smoke_camera(width, spp, depth=12):
    return scenes.cornell_camera(width, 1, depth).with_pixel_sample_mode(abi.GT_SAMPLE_RANDOM).with_samples_per_pixel(spp)


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("mode", ["plain", "mixture", "nee"])
def test_media_smoke_scene(gpu_context, precision, mode):
    # cornell_smoke_world (raytracing/scenes.rs:296-378): two ConstantMedium boxes under
    # RotateY / Translate after the walls.  Each ray's media draw from the pixel's stream
    # after its surfaces (scene.rs:177-197, medium.rs:170-187), next-event shadow rays
    # included (camera.rs:2248), so the f64 image matches the oracle's only if every draw
    # lands where the reference takes it.
    scene, lights = scenes.cornell_smoke_scene()
    cam = _smoke_camera(40, 6)
    if mode == "nee":
        cam = cam.with_direct_lighting_mode(abi.GT_DIRECT_NEXT_EVENT_ESTIMATION)
    use = None if mode == "plain" else lights
    pt = PathTracer(cam, precision=precision, context=gpu_context)
    render = (lambda **k: pt.render_hdr_image(scene, **k)) if use is None else \
        (lambda **k: pt.render_with_lights_hdr_image(scene, use, **k))
    ref, acc = _oracle_render(scene, cam, use)
    if precision == "f64":
        img = render(want64=True)
        np.testing.assert_array_equal(img.accepted, acc)
        err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
        assert (err <= 1e-9).mean() >= 0.99, err.max()
    else:
        img = render()
        ref32, _ = _oracle_render(scene, cam, use, precision=0)
        assert_explained(f"smoke {mode}", scene, cam, img.pixels, ref, ref32, use)
    st = pt.last_stats  # every ray ran in the persistent kernel's media variant
    assert st["persistent_rays"] == st["rays"] + st["shadow_rays"]
    assert (st["shadow_rays"] > 0) == (mode == "nee")
    assert np.isfinite(img.pixels).all()


def test_media_phase_function_environment_and_aovs(gpu_context):
    # A sphere-bounded Henyey-Greenstein medium, a plain sphere medium and an environment
    # light: the environment's shadow query (occlusion) draws for the media too
    # (camera.rs:2284-2290); the denoising AOVs draw from the same stream (camera.rs:3104).
    from gartus_gb300.raytracing import MediumBoundary
    scene = RayScene()
    ground = scene.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    scene.add_sphere((0.0, -100.5, -1.0), 100.0, ground)
    scene.add_sphere((1.1, 0.0, -1.3), 0.45, scene.add_material(RayMaterial.metal((0.8, 0.8, 0.8), 0.1)))
    scene.add_medium_with_phase_function(MediumBoundary.sphere((-0.6, 0.1, -1.2), 0.6), 1.5,
                                         RayMaterial.henyey_greenstein((0.9, 0.8, 0.7), 0.5))
    scene.add_constant_medium(MediumBoundary.box((-0.3, -0.5, -2.6), (0.5, 0.6, -1.8)).rotate_y(25.0),
                              3.0, (0.4, 0.6, 0.9))
    scene.build_bvh()
    env = EnvironmentLight(_env_u8(7, 16, 8))
    cam = RayCamera(40, 1.5).with_samples_per_pixel(6).with_max_depth(10)
    img = PathTracer(cam, precision="f64", context=gpu_context).render_with_environment_hdr_image(
        scene, env, want64=True)
    ref, acc = _oracle_render(scene, cam, env=env)
    np.testing.assert_array_equal(img.accepted, acc)
    err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
    assert (err <= 1e-9).mean() >= 0.99, err.max()
    aovs = PathTracer(cam, precision="f64", context=gpu_context).render_denoising_aovs(scene)
    _, _, alb, nrm = _oracle_render(scene, cam, aovs=True)
    np.testing.assert_allclose(aovs.albedo_linear, alb, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(aovs.normal_linear, nrm, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_media_batch_and_unsupported(gpu_context, precision):
    # A batch of a scene with media runs the persistent batch (MEDIA variant) and gives
    # each frame's single render; accumulation of such a scene is refused.
    from gartus_gb300.raytracing import Accumulator
    scene, lights = scenes.cornell_smoke_scene()
    cams = [_smoke_camera(24, 3).with_rng_seed(s) for s in (1, 2)] + [_smoke_camera(16, 2)]
    pt = PathTracer(cams[0], precision=precision, context=gpu_context)
    imgs = pt.render_batch_hdr_images(scene, cams, lights=lights, want64=precision == "f64")
    for cam, img in zip(cams, imgs):
        one = PathTracer(cam, precision=precision, context=gpu_context).render_with_lights_hdr_image(
            scene, lights, want64=precision == "f64")
        np.testing.assert_array_equal(img.accepted, one.accepted)
        if precision == "f64":
            np.testing.assert_array_equal(img.pixels64, one.pixels64)
        else:
            assert_modes_agree("media batch frame vs single frame", scene, cam, img.pixels, one.pixels, lights)
    # accumulation: 3 + 5 samples on one accumulator give the 8-sample render (the streams
    # continue in the persistent kernel's world variant)
    base = _smoke_camera(24, 1)
    full = PathTracer(base.with_samples_per_pixel(8), precision=precision, context=gpu_context
                      ).render_with_lights_hdr_image(scene, lights, want64=precision == "f64")
    acc = Accumulator(24, 24, precision, gpu_context)
    pt = PathTracer(base, context=gpu_context)
    pt.render_accumulate(scene, acc, 3, lights=lights)
    img = pt.render_accumulate(scene, acc, 5, lights=lights)
    assert acc.samples == 8
    np.testing.assert_array_equal(img.accepted, full.accepted)
    if precision == "f64":
        np.testing.assert_array_equal(img.pixels64, full.pixels64)
    else:
        assert_modes_agree("media accumulated vs one render", scene, base.with_samples_per_pixel(8), img.pixels,
                           full.pixels, lights)


def _bouncing_spheres(frame: int, n: int = 300):
    """Frame `frame` of a small animation: n spheres on a floor, each moving on its own
    seeded path (the dynamic layer), plus the floor (static)."""
    rng = np.random.default_rng(17)
    base = rng.uniform((-4, 0.2, -6), (4, 2.5, -1), size=(n, 3))
    vel = rng.normal(size=(n, 3)) * 0.15
    scene = RayScene()
    floor = scene.add_material(RayMaterial.checker_lambertian(0.5, (0.2, 0.3, 0.1), (0.9, 0.9, 0.9)))
    mats = [scene.add_material(RayMaterial.lambertian(tuple(rng.uniform(0.1, 0.9, 3)))) for _ in range(4)]
    mats.append(scene.add_material(RayMaterial.metal((0.8, 0.8, 0.8), 0.05)))
    light = scene.add_material(RayMaterial.diffuse_light((6.0, 6.0, 6.0)))
    scene.add_quad((-10.0, 0.0, 2.0), (20.0, 0.0, 0.0), (0.0, 0.0, -14.0), floor)
    scene.add_quad((-2.0, 6.0, -5.0), (4.0, 0.0, 0.0), (0.0, 0.0, 3.0), light)
    for i in range(n):
        c = base[i] + vel[i] * frame
        c[1] = abs(c[1] - 0.2) + 0.2  # bounce off the floor
        scene.add_sphere(tuple(c), 0.15 + 0.05 * (i % 3), mats[i % len(mats)])
    scene.build_bvh()
    return scene


@pytest.mark.parametrize("builder", ["gpu", "reference"])
def test_update_primitives_refit(gpu_context, builder):
    # gt_scene_update_primitives moves the dynamic spheres in place between frames.  With
    # the GPU-built tree the f32 path refits it on the device; the image then agrees with a
    # scene built from scratch at that frame, and the f64 path (reference tree rebuilt on
    # the host) with the oracle.
    cam = RayCamera(48, 1.5).with_samples_per_pixel(4).with_max_depth(6).with_look_at((0.0, 2.0, 4.0), (0.0, 1.0, -3.0))
    scene = _bouncing_spheres(0)
    if builder == "gpu":
        scene.use_gpu_bvh()
    pt32 = PathTracer(cam, context=gpu_context)
    pt64 = PathTracer(cam, precision="f64", context=gpu_context)
    pt32.render_hdr_image(scene)  # both copies resident before the updates
    pt64.render_hdr_image(scene, want64=True)
    for frame in (1, 2, 5):
        fresh = _bouncing_spheres(frame)
        if builder == "gpu":
            fresh.use_gpu_bvh()
        moved = fresh.primitives_array()[2:]
        scene.update_primitives(2, moved)
        np.testing.assert_array_equal(scene.primitives_array(), fresh.primitives_array())
        a = pt32.render_hdr_image(scene)
        b = PathTracer(cam, context=gpu_context).render_hdr_image(fresh)
        assert_modes_agree(f"refit frame {frame} vs rebuilt", fresh, cam, a.pixels, b.pixels)
        img64 = pt64.render_hdr_image(scene, want64=True)
        ref, acc = _oracle_render(fresh, cam)
        np.testing.assert_array_equal(img64.accepted, acc)
        err = rel_err(img64.pixels64, ref, floor=1e-12).max(axis=2)
        assert (err <= 1e-9).mean() >= 0.99
        assert scene.bvh_node_count(gpu_context) == fresh.bvh_node_count(gpu_context)
    with pytest.raises(ValueError):
        scene.update_primitives(len(scene.primitives_array()), scene.primitives_array()[:1])
    bad = scene.primitives_array()[:1].copy()
    bad["material"] = 99
    with pytest.raises(ValueError):
        scene.update_primitives(0, bad)
    with pytest.raises(GartusError):  # the library checks the range itself
        check(lib().gt_scene_update_primitives(scene._handle(gpu_context).h, 10**6, 1,
                                               scene.primitives_array()[:1].ctypes.data_as(C.c_void_p)))


def _uv_sphere(center, radius, rings=8, segs=12):
    """A tessellated sphere: (N, 3, 3) triangles with per-vertex texture coordinates
    (N, 3, 2) and smooth vertex normals (N, 3, 3)."""
    tris, uvs, nrms = [], [], []

    def vert(i, j):
        th, ph = math.pi * i / rings, 2 * math.pi * j / segs
        n = np.array([math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph)])
        return np.asarray(center) + radius * n, (j / segs, 1.0 - i / rings), n

    for i in range(rings):
        for j in range(segs):
            a, b, c, d = vert(i, j), vert(i + 1, j), vert(i + 1, j + 1), vert(i, j + 1)
            for t in ((a, b, c), (a, c, d)):
                tris.append([v[0] for v in t])
                uvs.append([v[1] for v in t])
                nrms.append([v[2] for v in t])
    return np.array(tris), np.array(uvs), np.array(nrms)


def _mesh_world():
    from gartus_gb300.raytracing import ImageTexture, MatrixInstance, NormalMap, TriangleMesh
    rng = np.random.default_rng(23)
    scene = RayScene()
    floor = scene.add_material(RayMaterial.lambertian((0.6, 0.6, 0.6)))
    light = scene.add_material(RayMaterial.diffuse_light((8.0, 8.0, 8.0)))
    scene.add_quad((-6.0, -0.6, 2.0), (12.0, 0.0, 0.0), (0.0, 0.0, -12.0), floor)
    scene.add_quad((-1.5, 3.5, -3.5), (3.0, 0.0, 0.0), (0.0, 0.0, 2.0), light)
    bumps = rng.integers(60, 196, size=(8, 8, 3), dtype=np.uint8)
    bumps[..., 2] = 230
    tex = ImageTexture(rng.integers(0, 256, size=(6, 9, 3), dtype=np.uint8), filter="linear", wrap_s="repeat")
    tris, uv, nrm = _uv_sphere((0.0, 0.0, 0.0), 0.6)
    bumpy = TriangleMesh(tris, RayMaterial.textured_lambertian(tex).with_normal_map(
        NormalMap(ImageTexture(bumps, filter="linear"), strength=1.5)), texcoords=uv, normals=nrm)
    smooth = TriangleMesh(tris, RayMaterial.ggx_microfacet((0.9, 0.8, 0.6), 0.25).with_normal_map(
        NormalMap(ImageTexture(bumps), flip_y=True)), texcoords=uv, normals=nrm,
        present=np.where(np.arange(len(tris)) % 5 == 0, 1, 3))
    ball = TriangleMesh.from_geometry([RayGeometry.sphere((0.0, 0.0, 0.0), 0.5)], RayMaterial.metal((0.9, 0.9, 0.9), 0.05))

    def trs(t, deg, scale):
        c, s = math.cos(math.radians(deg)), math.sin(math.radians(deg))
        m = np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1.0]]) @ np.diag(list(scale) + [1.0])
        m[:3, 3] = t
        return m

    scene.add_object(TriangleMesh(tris + np.array([-1.4, 0.0, -3.0]), bumpy.material, texcoords=uv, normals=nrm))
    scene.add_object(MatrixInstance(bumpy, trs((0.0, 0.0, -3.2), 30.0, (1.0, 1.0, 1.0))))
    scene.add_object(MatrixInstance(smooth, trs((1.4, 0.1, -3.0), -20.0, (1.2, 0.8, 1.0))))
    scene.add_object(TriangleMesh(tris + np.array([0.7, 0.9, -4.2]), smooth.material, texcoords=uv, normals=nrm))
    scene.add_object(MatrixInstance(ball, trs((-0.6, -0.1, -2.0), 0.0, (1.0, 0.5, 1.0))))
    scene.build_bvh()
    lights = SamplingTargetList()
    lights.add_quad((-1.5, 3.5, -3.5), (3.0, 0.0, 0.0), (0.0, 0.0, 2.0))
    return scene, lights


@pytest.mark.parametrize("schedule", ["wavefront", "persistent"])
@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("mode", ["mixture", "nee"])
def test_meshes_and_instances(gpu_context, precision, mode, schedule):
    # TriangleMesh with texture coordinates, vertex normals and normal maps (mesh.rs:56-141,
    # material.rs:1663-1684) and MatrixInstance (instance.rs:205-317) placing meshes and a
    # sphere, after the RayScene's surfaces: the f64 image matches the oracle's, on the
    # wavefront (whose kernels test the objects after the RayScene) and in the persistent
    # kernel's world variant.
    scene, lights = _mesh_world()
    cam = (RayCamera(48, 1.5).with_samples_per_pixel(4).with_max_depth(8)
           .with_look_at((0.0, 1.0, 2.0), (0.0, 0.0, -3.0)).with_background((0.1, 0.1, 0.12)))
    if mode == "nee":
        cam = cam.with_direct_lighting_mode(abi.GT_DIRECT_NEXT_EVENT_ESTIMATION)
    pt = PathTracer(cam, precision=precision, context=gpu_context, schedule=schedule)
    ref, acc = _oracle_render(scene, cam, lights)
    if precision == "f64":
        img = pt.render_with_lights_hdr_image(scene, lights, want64=True)
        np.testing.assert_array_equal(img.accepted, acc)
        err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
        assert (err <= 1e-9).mean() >= 0.99, err.max()
    else:
        img = pt.render_with_lights_hdr_image(scene, lights)
        ref32, _ = _oracle_render(scene, cam, lights, precision=0)
        assert_explained(f"meshes {mode} {schedule}", scene, cam, img.pixels, ref, ref32, lights)
    st = pt.last_stats
    assert st["persistent_rays"] == (st["rays"] + st["shadow_rays"] if schedule == "persistent" else 0)
    assert (st["shadow_rays"] > 0) == (mode == "nee")
    assert np.std(ref) > 1e-3


@pytest.mark.parametrize("mode", ["mixture", "nee"])
def test_object_world_schedules_agree(gpu_context, mode):
    # A world with objects and no media: the wavefront (one or three stripes), the automatic
    # schedule (the wavefront, then its last slots in the world variant of the persistent
    # kernel) and the persistent kernel evaluate the same arithmetic in the same order, so
    # the f64 images and the ray counts are identical; 2 + 2 accumulated samples (which run
    # on the wavefront too) give the 4-sample render.
    from gartus_gb300.raytracing import Accumulator
    scene, lights = _mesh_world()
    cam = (RayCamera(64, 1.5).with_samples_per_pixel(4).with_max_depth(8)
           .with_look_at((0.0, 1.0, 2.0), (0.0, 0.0, -3.0)).with_background((0.1, 0.1, 0.12)))
    if mode == "nee":
        cam = cam.with_direct_lighting_mode(abi.GT_DIRECT_NEXT_EVENT_ESTIMATION)
    runs = {}
    for name, kw in (("persistent", dict(schedule="persistent")), ("wavefront", dict(schedule="wavefront")),
                     ("stripes", dict(schedule="wavefront", stripes=3)), ("auto", dict(tail_slots=1000))):
        pt = PathTracer(cam, precision="f64", context=gpu_context, **kw)
        runs[name] = (pt.render_with_lights_hdr_image(scene, lights, want64=True), dict(pt.last_stats))
    img0, st0 = runs["persistent"]
    for name in ("wavefront", "stripes", "auto"):
        img, st = runs[name]
        np.testing.assert_array_equal(img.pixels64, img0.pixels64)
        np.testing.assert_array_equal(img.accepted, img0.accepted)
        for key in ("samples", "rays", "shadow_rays"):
            assert st[key] == st0[key], (name, key, st[key], st0[key])
    assert runs["wavefront"][1]["persistent_rays"] == 0
    assert 0 < runs["auto"][1]["persistent_rays"] < runs["auto"][1]["rays"] + runs["auto"][1]["shadow_rays"]
    acc = Accumulator(64, 42, "f64", gpu_context)
    pt = PathTracer(cam.with_samples_per_pixel(2), precision="f64", context=gpu_context)
    pt.render_accumulate(scene, acc, 2, lights=lights)
    two = pt.render_accumulate(scene, acc, 2, lights=lights)
    np.testing.assert_array_equal(two.pixels64, img0.pixels64)
    np.testing.assert_array_equal(two.accepted, img0.accepted)


def test_object_meshes_wide_and_binary_trees(gpu_context):
    # In f32 each object's mesh is walked through its eight-wide tree (the RayScene's walk,
    # traverse_wide); with binary f32 trees requested it keeps the reference tree.  The two
    # f32 images agree within the f32 tolerance, and the wide one is explained against the
    # oracle by test_meshes_and_instances.
    wide, lights = _mesh_world()
    binary, _ = _mesh_world()
    binary.use_binary_f32_tree(True)
    cam = (RayCamera(64, 1.5).with_samples_per_pixel(4).with_max_depth(8)
           .with_look_at((0.0, 1.0, 2.0), (0.0, 0.0, -3.0)).with_background((0.1, 0.1, 0.12))
           .with_direct_lighting_mode(abi.GT_DIRECT_NEXT_EVENT_ESTIMATION))
    a = PathTracer(cam, context=gpu_context).render_with_lights_hdr_image(wide, lights)
    b = PathTracer(cam, context=gpu_context).render_with_lights_hdr_image(binary, lights)
    assert_modes_agree("object meshes: wide vs binary f32 trees", wide, cam, a.pixels, b.pixels, lights)


def test_meshes_aovs_batch_and_primary(gpu_context):
    # The AOVs read the shading normal (camera.rs:3112-3114); a batch of an object world runs
    # on the wavefront (f32 frames of one width; its OBJ kernels in BATCH mode) or the
    # persistent batch (f64), and each frame equals its single render; gt_trace_rays sees
    # the RayScene only, as RayScene::hit does.
    scene, lights = _mesh_world()
    cam = RayCamera(40, 1.5).with_samples_per_pixel(3).with_max_depth(6).with_look_at((0.0, 1.0, 2.0), (0.0, 0.0, -3.0))
    aovs = PathTracer(cam, precision="f64", context=gpu_context).render_denoising_aovs(scene)
    _, _, alb, nrm = _oracle_render(scene, cam, aovs=True)
    np.testing.assert_allclose(aovs.albedo_linear, alb, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(aovs.normal_linear, nrm, rtol=1e-6, atol=1e-6)
    cams = [cam.with_rng_seed(5), cam.with_samples_per_pixel(2)]
    for precision in ("f64", "f32"):
        imgs = PathTracer(cam, precision=precision, context=gpu_context).render_batch_hdr_images(
            scene, cams, lights=lights, want64=precision == "f64")
        for c, img in zip(cams, imgs):
            one = PathTracer(c, precision=precision, context=gpu_context).render_with_lights_hdr_image(
                scene, lights, want64=precision == "f64")
            if precision == "f64":
                np.testing.assert_array_equal(img.pixels64, one.pixels64)
            else:
                assert_modes_agree("object-world batch frame vs single frame", scene, c, img.pixels, one.pixels, lights)
    rays = np.zeros((64, 7))
    rays[:, :3] = (0.0, 1.0, 2.0)
    rays[:, 3:6] = np.random.default_rng(4).normal(size=(64, 3)) * 0.3 + (0.0, -0.2, -1.0)
    ids, _, _ = scene.hit_rays(rays, ctx=gpu_context)
    assert set(np.unique(ids)) <= {-1, 0, 1} and (ids == 0).any()  # the floor and light quads only


def test_world_edge_cases(gpu_context):
    # Objects and media together (objects before media in the hit order), an empty mesh
    # placed twice, a texture-coordinate-only mesh with an image texture, and invalid
    # world descriptions refused by the library.
    from gartus_gb300.raytracing import ImageTexture, MatrixInstance, MediumBoundary, TriangleMesh, _SceneHandle
    tris, uv, _ = _uv_sphere((0.0, 0.0, -2.5), 0.7, 6, 10)
    scene = RayScene()
    scene.add_quad((-4.0, -0.8, 1.0), (8.0, 0.0, 0.0), (0.0, 0.0, -8.0), scene.add_material(RayMaterial.lambertian((0.7,) * 3)))
    tex = ImageTexture(np.random.default_rng(2).integers(0, 256, size=(4, 4, 3), dtype=np.uint8))
    scene.add_object(TriangleMesh(tris, RayMaterial.textured_lambertian(tex), texcoords=uv))
    empty = TriangleMesh(np.zeros((0, 3, 3)), RayMaterial.lambertian((0.5,) * 3))
    scene.add_object(empty)
    scene.add_object(MatrixInstance(empty, np.eye(4)))
    scene.add_constant_medium(MediumBoundary.sphere((0.0, 0.0, -2.5), 1.2), 0.6, (0.8, 0.8, 0.9))
    scene.build_bvh()
    cam = RayCamera(32, 1.5).with_samples_per_pixel(4).with_max_depth(8).with_background((0.6, 0.7, 0.9))
    img = PathTracer(cam, precision="f64", context=gpu_context).render_hdr_image(scene, want64=True)
    ref, acc = _oracle_render(scene, cam)
    np.testing.assert_array_equal(img.accepted, acc)
    err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
    assert (err <= 1e-9).mean() >= 0.99, err.max()
    # invalid: an object naming a missing mesh, a normal map on a metal, an image index past the table
    prims, mats = scene.primitives_array(), scene.materials_array()
    meshes, objects = scene.mesh_list(), scene.object_list()
    with pytest.raises(GartusError):
        _SceneHandle(gpu_context, prims, mats, 4, abi.GT_BVH_REFERENCE_SAH, scene.images(), (), meshes, [(7, None, None)])
    bad = mats.copy()
    bad[0]["kind"] = abi.GT_MAT_METAL
    bad[0]["normal_map"] = 1
    with pytest.raises(GartusError):
        _SceneHandle(gpu_context, prims, bad, 4, abi.GT_BVH_REFERENCE_SAH, scene.images(), (), meshes, objects)
    bad = mats.copy()
    bad[0]["normal_map"] = 9
    with pytest.raises(GartusError):
        _SceneHandle(gpu_context, prims, bad, 4, abi.GT_BVH_REFERENCE_SAH, scene.images(), (), meshes, objects)
    # a world with objects and media accumulates: 2 + 2 samples give the 4-sample render
    from gartus_gb300.raytracing import Accumulator
    acc_obj = Accumulator(32, 21, "f64", gpu_context)
    pt = PathTracer(cam.with_samples_per_pixel(1), context=gpu_context)
    pt.render_accumulate(scene, acc_obj, 2)
    two = pt.render_accumulate(scene, acc_obj, 2)
    np.testing.assert_array_equal(two.pixels64, img.pixels64)
