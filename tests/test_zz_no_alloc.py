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
from gartus_gb300.raytracing import PathTracer, RayMaterial, RayScene
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def _call(ctx, scene, lights, cam, rgb_ptr, acc_ptr):
    return lib().gt_render_noalloc(scene._handle(ctx).h, lights._handle(ctx).h if lights is not None else None,
                                   None, C.byref(cam.desc()), rgb_ptr, acc_ptr)


def test_noalloc_matches_gt_render_on_two_calls_in_a_row(gpu_context):
    import torch

    scene, lights = scenes.cornell_scene()
    cam = scenes.cornell_camera(96, 4, 50)
    # Set-up with the allocating entry point: makes scene and lights resident in f32 and
    # gives the reference image.
    ref = PathTracer(cam, context=gpu_context, schedule="persistent").render_with_lights_hdr_image(scene, lights)
    w, h, _ = cam.image_size()
    dev = torch.device(f"cuda:{gpu_context.device}")
    rgb = torch.full((h, w, 3), float("nan"), dtype=torch.float32, device=dev)
    acc = torch.zeros((h, w), dtype=torch.int32, device=dev)
    torch.cuda.synchronize(dev)
    assert _call(gpu_context, scene, lights, cam, rgb.data_ptr(), acc.data_ptr()) == abi.GT_OK
    free_after_first = torch.cuda.mem_get_info(dev)[0]
    for call in range(2):
        rgb.fill_(float("nan"))
        acc.zero_()
        torch.cuda.synchronize(dev)
        assert _call(gpu_context, scene, lights, cam, rgb.data_ptr(), acc.data_ptr()) == abi.GT_OK, \
            lib().gt_last_error()
        out = rgb.cpu().numpy()
        assert np.isfinite(out).all()
        np.testing.assert_array_equal(acc.cpu().numpy().astype(np.uint32), ref.accepted)
        # The f32 tolerance used for f32 comparisons elsewhere: pixels beyond 1e-4 relative
        # only where f32 rounding flipped a decision.
        err = rel_err(out, ref.pixels, floor=1e-3).max(axis=2)
        assert (err > 1e-4).sum() <= 0.02 * err.size, call
    # Nothing was allocated by the repeated calls.
    assert torch.cuda.mem_get_info(dev)[0] == free_after_first


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
