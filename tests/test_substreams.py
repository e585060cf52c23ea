"""The throughput mode (gt_render_opts.rng = GT_RNG_SUBSTREAMS; no reference counterpart).

Sample s of pixel (x, y) draws from its own SplitMix64 stream started at
pixel_seed(seed, x, y) ^ sample_key(s) instead of continuing the pixel's one stream
(raytracing/camera.rs:2669), so every (pixel, sample) pair is a work item.  The oracle
renders the same mode (oracle.OracleScene.render(rng="substreams"): the same restatement
of the reference, with the per-sample streams), so the checks of the reference mode apply
unchanged: f64 pixels to 1e-9 with equal accepted counts, every f32 pixel beyond 1e-4
explained by a decision flip or f32 drift, and (check 3) the converged image within the
f64 oracle's own noise floor of the reference's pixel-stream image."""
import ctypes as C

import numpy as np
import pytest

import oracle
from gartus_gb300 import abi, scenes
from gartus_gb300._lib import GartusError
from gartus_gb300.raytracing import Accumulator, PathTracer, RayCamera
from tests.divergence import assert_explained, assert_modes_agree
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def _oracle(scene, cam, lights=None, env=None, precision=1, rng="substreams"):
    o = oracle.OracleScene.from_ray_scene(scene)
    la = lights.to_array() if lights is not None else None
    return o.render(cam.desc(), la, env, precision=precision, threads=8, rng=rng)


def _render(pt, scene, lights=None, env=None, want64=False):
    if env is not None:
        return pt.render_with_environment_hdr_image(scene, env, want64=want64)
    if lights is not None:
        return pt.render_with_lights_hdr_image(scene, lights, want64=want64)
    return pt.render_hdr_image(scene, want64=want64)


def _cases():
    final = scenes.final_scene_ray_scene()
    cornell, lights = scenes.cornell_scene()
    batch, blights = scenes.batch_scene()
    mesh, env = scenes.mesh_heavy_scene(size=40, tori=6, rings=8, tube=12, env_width=256, env_height=128)
    from tests.test_gpu_parity import _mesh_world
    objects, olights = _mesh_world()
    return {
        # random sampling with defocus; 512 x 288 x 128 spp (18.9 M samples) spans several
        # rounds of (pixel, sample) items
        "final_rounds": (final, scenes.final_scene_camera(512, 128), None, None),
        "cornell_mixture": (cornell, scenes.cornell_camera(40, 3, 50), lights, None),
        "cornell_nee": (cornell, scenes.cornell_camera(32, 2, 50).with_direct_lighting_mode(
            abi.GT_DIRECT_NEXT_EVENT_ESTIMATION), lights, None),
        # adaptive random sampling (minimum 8, cap 64) with motion blur
        "adaptive": (batch, scenes.batch_cameras(frames=3, width=40, spp_cycle=(8,), max_samples=64,
                                                 threshold=0.05)[1], blights, None),
        "environment": (mesh, scenes.mesh_heavy_camera(48, 27, 3, 8), None, env),
        # meshes and instances (a world with objects: the wavefront's OBJ kernels), NEE
        "objects": (objects, RayCamera(48, 1.5).with_samples_per_pixel(6).with_max_depth(8)
                    .with_look_at((0.0, 1.0, 2.0), (0.0, 0.0, -3.0)).with_background((0.1, 0.1, 0.12))
                    .with_direct_lighting_mode(abi.GT_DIRECT_NEXT_EVENT_ESTIMATION), olights, None),
    }


@pytest.mark.parametrize("case", ["final_rounds", "cornell_mixture", "cornell_nee", "adaptive", "environment",
                                  "objects"])
def test_f64_substreams_match_oracle(gpu_context, case):
    scene, cam, lights, env = _cases()[case]
    pt = PathTracer(cam, precision="f64", context=gpu_context, rng="substreams")
    img = _render(pt, scene, lights, env, want64=True)
    ref, acc = _oracle(scene, cam, lights, env)
    np.testing.assert_array_equal(img.accepted, acc)
    err = rel_err(img.pixels64, ref, floor=1e-12).max(axis=2)
    print(f"{case}: f64 substreams max relative error {err.max():.3e}, {pt.last_stats['iterations']} iterations")
    assert err.max() <= 1e-9
    # the streams are the mode's own, not the reference's
    ref_pixel, _ = _oracle(scene, cam, lights, env, rng="pixel")
    assert not np.array_equal(ref, ref_pixel)


@pytest.mark.parametrize("case", ["final_rounds", "cornell_mixture", "cornell_nee", "adaptive", "environment",
                                  "objects"])
def test_f32_substreams_explained(gpu_context, case):
    scene, cam, lights, env = _cases()[case]
    pt = PathTracer(cam, context=gpu_context, rng="substreams")
    img = _render(pt, scene, lights, env)
    ref64, acc = _oracle(scene, cam, lights, env)
    ref32, _ = _oracle(scene, cam, lights, env, precision=0)
    assert_explained(f"substreams {case}", scene, cam, img.pixels, ref64, ref32, lights, env, rng="substreams")
    flipped = int((img.accepted != acc).sum())  # adaptive stops may flip in f32
    assert flipped <= 0.02 * acc.size, flipped
    # reproducible: the fold adds each pixel's samples in sample order
    again = _render(pt, scene, lights, env)
    np.testing.assert_array_equal(again.pixels, img.pixels)


def test_substream_stripes_and_engines_agree(gpu_context):
    # The wavefront engine deals a round's sample rows to stripes; every slot runs the same
    # arithmetic whichever stripe holds it and the fold adds samples in sample order, so
    # the image does not depend on the stripe count (1, 2 and 3 stripes over the 128
    # sample rows of an 80 x 45 frame; 3 leaves the stripes uneven).
    final = scenes.final_scene_ray_scene()
    cam = scenes.final_scene_camera(80, 128)
    imgs = [PathTracer(cam, context=gpu_context, rng="substreams", stripes=k).render_hdr_image(final)
            for k in (1, 2, 3)]
    for img in imgs[1:]:
        np.testing.assert_array_equal(img.pixels, imgs[0].pixels)
        np.testing.assert_array_equal(img.accepted, imgs[0].accepted)


def test_substreams_converge_to_the_reference(gpu_context):
    # Check 3 at 576 spp: the f32 substream image's relMSE against an f64 image of the
    # reference's own streams is no larger than the noise floor between two such images.
    scene, lights = scenes.cornell_scene()
    cam = scenes.cornell_camera(24, 24, 50)
    img = PathTracer(cam, context=gpu_context, rng="substreams").render_with_lights_hdr_image(scene, lights)
    x = img.pixels.astype(np.float64)
    ref, _ = _oracle(scene, cam, lights, rng="pixel")
    other, _ = _oracle(scene, cam.with_rng_seed(12345), lights, rng="pixel")
    rel = lambda a, b: float(np.mean((a - b) ** 2 / (b * b + 1e-2)))
    e_sub, e_floor = rel(x, ref), rel(other, ref)
    print(f"check 3: substreams f32 relMSE {e_sub:.3e} against the reference-stream f64 image; "
          f"f64 noise floor {e_floor:.3e}")
    assert e_sub <= 1.1 * e_floor + 1e-4


def test_substream_batch_equals_single_frames(gpu_context):
    # A batch in substream mode: the frames' pixels are one list of work items, whatever
    # their widths; each frame equals its own substream render.
    scene, lights = scenes.batch_scene()
    cams = scenes.batch_cameras(frames=4, width=40, spp_cycle=(4, 8), max_samples=32, threshold=0.05)
    cams.append(scenes.cornell_camera(24, 3, 20))  # another width, stratified
    pt = PathTracer(cams[0], context=gpu_context, rng="substreams")
    imgs = pt.render_batch_hdr_images(scene, cams, lights=lights)
    assert pt.last_stats["samples"] == sum(int(i.accepted.sum()) for i in imgs)
    for cam, img in zip(cams, imgs):
        one = PathTracer(cam, context=gpu_context, rng="substreams").render_with_lights_hdr_image(scene, lights)
        flipped = int((img.accepted != one.accepted).sum())
        assert flipped <= 0.02 * img.accepted.size, flipped
        assert_modes_agree("substream batch frame vs single frame", scene, cam, img.pixels, one.pixels, lights,
                           rng="substreams")


def test_substream_aovs_progress_and_cancel(gpu_context):
    # The AOV pass keeps the reference's per-pixel streams (render_denoising_aovs is its own
    # render in the reference), so the substream render's albedo and normal planes equal
    # the reference mode's; the beauty plane is the substream image.  Progress is reported
    # after every round with the image of the samples folded so far, and a callback that
    # cancels ends the render with GT_ERR_CANCELLED.
    scene = scenes.final_scene_ray_scene()
    cam = scenes.final_scene_camera(64, 8)
    sub = PathTracer(cam, context=gpu_context, rng="substreams").render_denoising_aovs(scene)
    ref = PathTracer(cam, context=gpu_context).render_denoising_aovs(scene)
    np.testing.assert_array_equal(sub.albedo_linear, ref.albedo_linear)
    np.testing.assert_array_equal(sub.normal_linear, ref.normal_linear)
    img = PathTracer(cam, context=gpu_context, rng="substreams").render_hdr_image(scene)
    np.testing.assert_array_equal(sub.beauty_linear, img.pixels)
    for engine_scene, engine_cam in ((scene, scenes.final_scene_camera(256, 256)),       # wavefront
                                     (scenes.cornell_scene()[0], scenes.cornell_camera(256, 16, 50))):  # k_substream
        seen, last = [], []
        pt = PathTracer(engine_cam, context=gpu_context, rng="substreams")
        img = pt.render_progressive(engine_scene,
                                    lambda u: (seen.append((u.completed, u.total)), last.append(u.pixels.copy())))
        assert seen and all(0 < c <= t for c, t in seen) and seen[-1][0] == seen[-1][1], seen
        assert np.isfinite(img.pixels).all()
        # the last progress image is the frame from every folded sample: the result
        np.testing.assert_array_equal(last[-1], img.pixels)

        class Stop(Exception):
            pass

        def stop(u):
            raise Stop()

        with pytest.raises(Stop):
            pt.render_progressive(engine_scene, stop)


def test_migrate_modes_keep_f64_images(gpu_context):
    # Migration is a scheduling choice: on, off and the default give the same f64 image
    # and accepted counts (Cornell at 64 spp per pixel, so that pixels migrate).
    scene, lights = scenes.cornell_scene()
    cam = scenes.cornell_camera(48, 8, 50)
    imgs = {m: PathTracer(cam, precision="f64", context=gpu_context, migrate=m).render_with_lights_hdr_image(
        scene, lights, want64=True) for m in ("default", "on", "off")}
    for m in ("on", "off"):
        np.testing.assert_array_equal(imgs[m].pixels64, imgs["default"].pixels64)
        np.testing.assert_array_equal(imgs[m].accepted, imgs["default"].accepted)
    with pytest.raises(ValueError):
        PathTracer(cam, migrate="sometimes")


def test_substream_unsupported_uses(gpu_context):
    scene, lights = scenes.cornell_scene()
    cam = scenes.cornell_camera(16, 1, 5)
    # accumulation continues the pixels' own streams
    acc = Accumulator(16, 16, context=gpu_context)
    with pytest.raises(GartusError, match="own streams"):
        PathTracer(cam.with_pixel_sample_mode(abi.GT_SAMPLE_RANDOM).with_samples_per_pixel(1), context=gpu_context,
                   rng="substreams").render_accumulate(scene, acc, 2, lights=lights)
    # batches render in f32
    with pytest.raises(GartusError, match="f32"):
        PathTracer(cam, precision="f64", context=gpu_context, rng="substreams").render_batch_hdr_images(
            scene, [cam, cam], lights=lights)
    # worlds with media, and batches of worlds with objects
    from tests.test_gpu_parity import _mesh_world
    objects, olights = _mesh_world()
    with pytest.raises(GartusError, match="substream batch"):
        PathTracer(cam, context=gpu_context, rng="substreams").render_batch_hdr_images(objects, [cam, cam],
                                                                                       lights=olights)
    smoke, _ = scenes.cornell_smoke_scene()
    with pytest.raises(GartusError, match="substreams"):
        PathTracer(cam, context=gpu_context, rng="substreams").render_hdr_image(smoke)
    with pytest.raises(ValueError):
        PathTracer(cam, rng="other")
    # an unknown mode through the C ABI
    o = abi.gt_render_opts()
    o.struct_size = C.sizeof(abi.gt_render_opts)
    o.rng = 7
    f = abi.gt_frame()
    f.struct_size = C.sizeof(abi.gt_frame)
    buf = np.zeros((16, 16, 3), dtype=np.float32)
    f.width, f.height, f.rgb = 16, 16, buf.ctypes.data
    from gartus_gb300._lib import lib
    st = lib().gt_render(scene._handle(gpu_context).h, lights._handle(gpu_context).h, None, C.byref(cam.desc()),
                         C.byref(o), C.byref(f))
    assert st == abi.GT_ERR_INVALID_ARG
