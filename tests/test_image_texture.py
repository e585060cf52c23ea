"""ImageTexture sampling in the oracle, pinned on the reference's texture tests
(graphics/texture.rs:911-952, graphics/raytracing.rs:607-620) and on a second, pure-Python
restatement of Texture::sample (graphics/texture.rs:696-752) for seeded random images."""
import math

import numpy as np
import pytest

import oracle
from gartus_gb300 import abi
from gartus_gb300.raytracing import ImageTexture, RayMaterial, RayScene

RED, GREEN, BLUE, WHITE = (255, 0, 0), (0, 255, 0), (0, 0, 255), (255, 255, 255)


def _tex(w, h, pixels, **kw):
    return ImageTexture(np.array(pixels, dtype=np.uint8).reshape(h, w, 3), **kw)


def _lin(rgb):
    return np.array([(c / 255.0) ** 2 for c in rgb])


def test_nearest_uses_bottom_left_origin():  # graphics/texture.rs:910-916
    t = _tex(2, 2, [RED, GREEN, BLUE, WHITE])
    np.testing.assert_array_equal(oracle.image_sample(t, 0.0, 0.0), _lin(BLUE))
    np.testing.assert_array_equal(oracle.image_sample(t, 1.0, 1.0), _lin(GREEN))


def test_repeat_wraps_coordinates():  # graphics/texture.rs:918-923
    t = _tex(2, 2, [RED, GREEN, BLUE, WHITE], wrap_s="repeat", wrap_t="repeat")
    np.testing.assert_array_equal(oracle.image_sample(t, 1.25, -0.25), oracle.image_sample(t, 0.25, 0.75))


def test_linear_blends_neighbours():  # graphics/texture.rs:925-940
    t = _tex(2, 2, [(0, 0, 0), (100, 0, 0), (0, 100, 0), (100, 100, 0)], filter="linear")
    np.testing.assert_array_equal(oracle.image_sample(t, 0.5, 0.5), _lin((50, 50, 0)))


def test_linear_repeat_wraps_across_seam():  # graphics/texture.rs:942-952
    t = _tex(2, 1, [RED, GREEN], filter="linear", wrap_s="repeat", wrap_t="repeat")
    c = oracle.image_sample(t, 0.99, 0.0)
    assert c[0] > c[1]


def test_image_texture_samples_bitmap():  # graphics/raytracing.rs:607-620
    t = _tex(2, 1, [RED, GREEN])
    np.testing.assert_array_equal(oracle.image_sample(t, 0.0, 0.5), [1.0, 0.0, 0.0])
    np.testing.assert_array_equal(oracle.image_sample(t, 1.0, 0.5), [0.0, 1.0, 0.0])


def test_empty_is_cyan_and_non_finite_is_black():  # raytracing/texture.rs:150-152, texture.rs:596-598
    np.testing.assert_array_equal(oracle.image_sample(ImageTexture(np.zeros((0, 0, 3), np.uint8)), 0.3, 0.3),
                                  [0.0, 1.0, 1.0])
    t = _tex(2, 1, [RED, GREEN])
    np.testing.assert_array_equal(oracle.image_sample(t, math.nan, 0.5), [0.0, 0.0, 0.0])
    np.testing.assert_array_equal(oracle.image_sample(t, 0.5, math.inf), [0.0, 0.0, 0.0])


def _sample_python(tex: ImageTexture, s: float, t: float) -> np.ndarray:
    """Texture::sample restated with Python floats: nearest rounds to the closest texel
    centre of [0, size - 1]; linear lerps u8 texels (Rgb::lerp rounds each channel)."""
    img = tex.texels.astype(np.int64)
    h, w = img.shape[:2]

    def wrap(x, mode):
        return x % 1.0 if mode == "repeat" else min(max(x, 0.0), 1.0)

    def lerp(a, b, f):
        f = min(max(f, 0.0), 1.0)
        return np.array([min(max(round_half_away(a[k] + (b[k] - a[k]) * f), 0), 255) for k in range(3)])

    if tex.filter == "nearest":
        x = int(round_half_away(wrap(s, tex.wrap_s) * (w - 1)))
        y = int(round_half_away((1.0 - wrap(t, tex.wrap_t)) * (h - 1)))
        c = img[y, x]
    else:
        def axis(v, size, mode):
            if mode == "clamp":
                coord = min(max(v, 0.0), 1.0) * (size - 1)
                lo = int(math.floor(coord))
                return coord, lo, min(lo + 1, size - 1)
            coord = (v % 1.0) * size
            lo = min(int(math.floor(coord)), size - 1)
            return coord, lo, 0 if lo + 1 == size else lo + 1

        x, x0, x1 = axis(s, w, tex.wrap_s)
        y, y0, y1 = axis(1.0 - t, h, tex.wrap_t)
        top = lerp(img[y0, x0], img[y0, x1], x - x0)
        bottom = lerp(img[y1, x0], img[y1, x1], x - x0)
        c = lerp(top, bottom, y - y0)
    return np.array([(v / 255.0) ** 2 for v in c])


def round_half_away(x: float) -> float:
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


@pytest.mark.parametrize("filter", ["nearest", "linear"])
@pytest.mark.parametrize("wrap", ["clamp", "repeat"])
def test_oracle_matches_python_restatement(filter, wrap):
    rng = np.random.default_rng(1234)
    for shape in ((1, 1), (1, 5), (4, 1), (7, 9), (16, 16)):
        tex = ImageTexture(rng.integers(0, 256, size=shape + (3,), dtype=np.uint8), filter=filter,
                           wrap_s=wrap, wrap_t="repeat" if wrap == "clamp" else "clamp")
        for s, t in rng.uniform(-2.5, 2.5, size=(60, 2)):
            np.testing.assert_array_equal(oracle.image_sample(tex, s, t), _sample_python(tex, s, t))


def test_scene_image_table_and_validation():
    a = ImageTexture(np.zeros((2, 3, 3), np.uint8))
    b = ImageTexture(np.full((1, 1, 3), 200, np.uint8), filter="linear")
    scene = RayScene()
    m0 = scene.add_material(RayMaterial.textured_lambertian(b))
    m1 = scene.add_material(RayMaterial.textured_lambertian(a))
    m2 = scene.add_material(RayMaterial.textured_diffuse_light(b))
    scene.add_sphere((0.0, 0.0, -1.0), 0.5, m0)
    assert scene.images() == [b, a]
    mats = scene.materials_array()
    assert [int(mats[i]["texture_kind"]) for i in (m0, m1, m2)] == [abi.GT_TEX_IMAGE] * 3
    assert [mats[i]["tex"][0] for i in (m0, m1, m2)] == [0.0, 1.0, 0.0]
    with pytest.raises(ValueError):
        ImageTexture(np.zeros((2, 2, 3), np.float32))
    with pytest.raises(ValueError):
        ImageTexture(np.zeros((2, 2, 3), np.uint8), filter="cubic")
    with pytest.raises(TypeError):
        RayMaterial.textured_lambertian(np.zeros((2, 2, 3), np.uint8))
    # the oracle rejects an image index past the table, as the library does
    bad = mats.copy()
    bad[0]["tex"][0] = 5.0
    with pytest.raises(ValueError):
        oracle.OracleScene(scene.primitives_array(), bad, 4, scene.images())
