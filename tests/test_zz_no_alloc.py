"""gt_render_noalloc: the render entry point for callers that cannot allocate device
memory while rendering (a real-time loop, a host runtime that owns all device memory).
It must give gt_render's image while allocating nothing, call after call.

This file runs last (pytest collects files in name order) so that a failure here leaves
every other test already run."""
import ctypes as C

import numpy as np
import pytest

from gartus_gb300 import abi, scenes
from gartus_gb300._lib import lib
from gartus_gb300.raytracing import EnvironmentLight, PathTracer, RayMaterial, RayScene

pytestmark = pytest.mark.gpu


def _call(ctx, scene, lights, cam, rgb_ptr, acc_ptr, env=None):
    return lib().gt_render_noalloc(scene._handle(ctx).h, lights._handle(ctx).h if lights is not None else None,
                                   env._handle(ctx).h if env is not None else None, C.byref(cam.desc()), rgb_ptr,
                                   acc_ptr)


def _twice(ctx, scene, lights, env, cam, ref):
    """Two calls in a row into one pair of device buffers; each must give `ref` (gt_render's
    persistent schedule runs the same kernels, so the images are identical) and the second
    allocates nothing."""
    import torch

    w, h, _ = cam.image_size()
    dev = torch.device(f"cuda:{ctx.device}")
    rgb = torch.full((h, w, 3), float("nan"), dtype=torch.float32, device=dev)
    acc = torch.zeros((h, w), dtype=torch.int32, device=dev)
    torch.cuda.synchronize(dev)
    assert _call(ctx, scene, lights, cam, rgb.data_ptr(), acc.data_ptr(), env) == abi.GT_OK, lib().gt_last_error()
    free_after_first = torch.cuda.mem_get_info(dev)[0]
    for call in range(2):
        rgb.fill_(float("nan"))
        acc.zero_()
        torch.cuda.synchronize(dev)
        assert _call(ctx, scene, lights, cam, rgb.data_ptr(), acc.data_ptr(), env) == abi.GT_OK, \
            lib().gt_last_error()
        out = rgb.cpu().numpy()
        assert np.isfinite(out).all()
        np.testing.assert_array_equal(acc.cpu().numpy().astype(np.uint32), ref.accepted)
        np.testing.assert_array_equal(out, ref.pixels)
    assert torch.cuda.mem_get_info(dev)[0] == free_after_first


def test_noalloc_matches_gt_render_on_two_calls_in_a_row(gpu_context):
    scene, lights = scenes.cornell_scene()
    cam = scenes.cornell_camera(96, 4, 50)
    # Set-up with the allocating entry point: makes scene and lights resident in f32 and
    # gives the reference image.
    ref = PathTracer(cam, context=gpu_context, schedule="persistent").render_with_lights_hdr_image(scene, lights)
    _twice(gpu_context, scene, lights, None, cam, ref)


def test_noalloc_media_world_and_environment(gpu_context):
    # The world variant (media after the surfaces) and an environment light through the
    # same fixed scratch.
    scene, lights = scenes.cornell_smoke_scene()
    cam = scenes.cornell_camera(32, 1, 20).with_pixel_sample_mode(abi.GT_SAMPLE_RANDOM).with_samples_per_pixel(3)
    ref = PathTracer(cam, context=gpu_context, schedule="persistent").render_with_lights_hdr_image(scene, lights)
    _twice(gpu_context, scene, lights, None, cam, ref)
    rng = np.random.default_rng(8)
    env = EnvironmentLight(rng.integers(0, 256, size=(8, 16, 3), dtype=np.uint8))
    scene = scenes.render_performance_scene()
    cam = scenes.render_performance_camera().with_samples_per_pixel(2)
    ref = PathTracer(cam, context=gpu_context, schedule="persistent").render_with_environment_hdr_image(scene, env)
    _twice(gpu_context, scene, None, env, cam, ref)


def test_noalloc_rejects_oversized_and_unprepared_inputs(gpu_context):
    import torch

    dev = torch.device(f"cuda:{gpu_context.device}")
    buf = torch.zeros(16, dtype=torch.float32, device=dev)
    scene, lights = scenes.cornell_scene()
    # Too many pixels for the fixed scratch array: a clear error, nothing launched.
    big = scenes.cornell_camera(1025, 1, 5)
    PathTracer(scenes.cornell_camera(8, 1, 5), context=gpu_context).render_with_lights_hdr_image(scene, lights)
    assert _call(gpu_context, scene, lights, big, buf.data_ptr(), None) == abi.GT_ERR_INVALID_ARG
    assert b"scratch" in lib().gt_last_error()
    # A scene that was never rendered is not resident; preparing it would allocate.
    fresh = RayScene()
    m = fresh.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    fresh.add_sphere((0.0, 0.0, -1.0), 0.5, m)
    cam = scenes.cornell_camera(4, 1, 5)
    assert _call(gpu_context, fresh, None, cam, buf.data_ptr(), None) == abi.GT_ERR_INVALID_ARG
    assert b"resident" in lib().gt_last_error()
