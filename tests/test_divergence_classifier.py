"""The f32 divergence classifier (tests/divergence.py) on the CPU, with the oracle standing
in for the GPU: the f32 oracle's own image is fully explained (every pixel it moves
beyond 1e-4 of f64 is a decision flip or continuous f32 drift), and mistakes planted in an
image on the CPU are caught: a pixel moved by 1% where neither a decision nor the f32
oracle explains it is unexplained, and small drifts are allowed on at most 0.5% of the
image."""
import numpy as np
import pytest

import oracle
from gartus_gb300 import abi, scenes
from tests.divergence import (GPU_ROUNDING, NEAR, UNEXPLAINED, assert_explained, classify, divergent_pixels,
                              MARGIN_TYPES)


@pytest.fixture(scope="module")
def cornell():
    scene, lights = scenes.cornell_scene()
    # few decisions per pixel (one sample, three bounces), so that many pixels have none
    # near its boundary
    cam = scenes.cornell_camera(40, 1, 3).with_direct_lighting_mode(abi.GT_DIRECT_NEXT_EVENT_ESTIMATION)
    o = oracle.OracleScene.from_ray_scene(scene)
    ref64, _ = o.render(cam.desc(), lights.to_array(), None, precision=1, threads=8)
    ref32, _ = o.render(cam.desc(), lights.to_array(), None, precision=0, threads=8)
    return scene, lights, cam, o, ref64, ref32


def _quiet_pixels(o, cam, lights, ref64, ref32, want):
    """Pixels where the f32 oracle stays within 1e-4 of f64 and no decision of the f64 run
    lies within NEAR of its boundary: a change there has no explanation but drift."""
    calm = ~divergent_pixels(ref32, ref64)
    out = []
    for y, x in np.argwhere(calm):
        t64 = o.pixel_trace(cam.desc(), int(x), int(y), lights.to_array(), None, precision=1)
        near = np.isin(t64[0], MARGIN_TYPES) & (np.abs(t64[2]) < NEAR)
        if not near.any() and np.abs(ref64[y, x]).max() > 1e-2:
            out.append((int(y), int(x)))
        if len(out) == want:
            break
    assert len(out) == want
    return out


@pytest.mark.parametrize("case", ["cornell_nee_depth50", "final_scene"])
def test_f32_oracle_image_is_explained(case):
    # Long paths and glass: the f32 oracle's image leaves f64 through decision flips and
    # drift, and the classifier names a cause for every such pixel.
    if case == "final_scene":
        scene, lights = scenes.final_scene_ray_scene(), None
        cam = scenes.final_scene_camera(48, 4)
    else:
        scene, lights = scenes.cornell_scene()
        cam = scenes.cornell_camera(24, 2, 50).with_direct_lighting_mode(abi.GT_DIRECT_NEXT_EVENT_ESTIMATION)
    o = oracle.OracleScene.from_ray_scene(scene)
    la = lights.to_array() if lights is not None else None
    ref64, _ = o.render(cam.desc(), la, None, precision=1, threads=8)
    ref32, _ = o.render(cam.desc(), la, None, precision=0, threads=8)
    counts = assert_explained(f"f32 oracle as the image ({case})", scene, cam, ref32, ref64, ref32, lights)
    assert UNEXPLAINED not in counts and GPU_ROUNDING not in counts
    assert sum(counts.values()) > 0  # the f32 oracle does leave f64 here


def test_planted_error_is_unexplained(cornell):
    scene, lights, cam, o, ref64, ref32 = cornell
    (y, x), = _quiet_pixels(o, cam, lights, ref64, ref32, 1)
    img = ref32.copy()
    img[y, x] = ref64[y, x] * 1.01
    counts, rows = classify(scene, cam, img, ref64, ref32, lights)
    assert [r[2] for r in rows if (r[0], r[1]) == (y, x)] == [UNEXPLAINED]
    with pytest.raises(AssertionError, match="unexplained"):
        assert_explained("planted 1% error", scene, cam, img, ref64, ref32, lights)


def test_small_drift_is_allowed_on_few_pixels_only(cornell):
    scene, lights, cam, o, ref64, ref32 = cornell
    total = ref64.shape[0] * ref64.shape[1]
    few = max(1, int(0.005 * total))
    pix = _quiet_pixels(o, cam, lights, ref64, ref32, few + 2)
    img = ref32.copy()
    for y, x in pix[:few]:  # within the GPU drift bound (1e-3), beyond the 1e-4 tolerance
        img[y, x] = ref64[y, x] * (1 + 5e-4)
    counts = assert_explained("drift on few pixels", scene, cam, img, ref64, ref32, lights)
    assert counts[GPU_ROUNDING] == few
    for y, x in pix[few:]:
        img[y, x] = ref64[y, x] * (1 + 5e-4)
    with pytest.raises(AssertionError, match="drift"):
        assert_explained("drift on too many pixels", scene, cam, img, ref64, ref32, lights)
