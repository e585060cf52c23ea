"""ConstantMedium in the oracle (raytracing/volume/medium.rs), pinned on the reference's
test (graphics/raytracing.rs:1065-1081), on a pure-Python restatement of the sphere-bounded
case, and on properties of box boundaries under RotateY / Translate (instance.rs)."""
import math

import numpy as np
import pytest

import oracle
from gartus_gb300 import scenes
from gartus_gb300.raytracing import MediumBoundary, RayMaterial, RayScene

INF = math.inf


def test_dense_medium_scatters_inside_boundary():  # graphics/raytracing.rs:1065-1081
    b = MediumBoundary.sphere((0.0, 0.0, -1.0), 0.5)
    t, draws = oracle.medium_hit(b, 1.0e9, [0, 0, 0, 0, 0, -1], 0.0, INF, 47)
    assert t is not None and 0.5 < t < 1.5
    assert draws == 1


def _sphere_roots(c, r, o, d):
    """hit_sphere_in_interval's two roots (object.rs:986-1013), or None."""
    oc = (c[0] - o[0], c[1] - o[1], c[2] - o[2])
    a = d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
    if a <= 2.220446049250313e-16:
        return None
    h = d[0] * oc[0] + d[1] * oc[1] + d[2] * oc[2]
    cc = (oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2]) - r * r
    disc = h * h - a * cc
    if disc < 0.0:
        return None
    sq = math.sqrt(disc)
    return (h - sq) / a, (h + sq) / a


def _first_root(roots, lo, hi):
    if roots is None:
        return None
    for x in roots:
        if lo < x < hi:
            return x
    return None


def _medium_python(c, r, density, o, d, tmin, tmax, seed):
    """ConstantMedium::hit_with_rng with a Sphere boundary, restated (medium.rs:119-187)."""
    roots = _sphere_roots(c, r, o, d)
    entry = _first_root(roots, -INF, INF)
    if entry is None:
        return None, 0
    entry = max(entry, tmin)
    exit_ = _first_root(roots, entry + 0.0001, INF)
    if exit_ is None:
        return None, 0
    exit_ = min(exit_, tmax)
    if entry >= exit_:
        return None, 0
    entry = max(entry, 0.0)
    length = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    if length <= 2.220446049250313e-16:
        return None, 0
    inside = (exit_ - entry) * length
    rng = scenes.SampleRng(seed)
    sample = max(rng.random_double(), 2.2250738585072014e-308)
    dist = (-1.0 / density) * math.log(sample)
    if dist > inside:
        return None, 1
    return entry + dist / length, 1


def test_sphere_medium_matches_python_restatement():
    rng = np.random.default_rng(5)
    hits = misses_after_draw = 0
    for _ in range(400):
        c = tuple(rng.uniform(-2, 2, 3))
        r = float(rng.uniform(0.2, 1.5))
        o = tuple(rng.uniform(-3, 3, 3))
        aim = np.array(c) + rng.normal(size=3) * r * 0.8  # mostly through the sphere
        d = tuple((aim - np.array(o)) * rng.uniform(0.3, 2.0))
        density = float(10 ** rng.uniform(-2, 1))
        tmax = INF if rng.random() < 0.7 else float(rng.uniform(0.0, 4.0))
        seed = int(rng.integers(0, 2**63))
        want = _medium_python(c, r, density, o, d, 0.001, tmax, seed)
        got = oracle.medium_hit(MediumBoundary.sphere(c, r), density, list(o) + list(d), 0.001, tmax, seed)
        assert got == want, (c, r, o, d, density, tmax)
        hits += want[0] is not None
        misses_after_draw += want[0] is None and want[1] == 1
    assert hits > 20 and misses_after_draw > 20


def test_box_medium_properties():
    # A translated, rotated box: rays that start outside and miss draw nothing; a ray aimed
    # through the box draws once and scatters between the entry and exit faces; an
    # interval clipped before the entry draws nothing; a dense medium scatters at entry.
    box = MediumBoundary.box((0.0, 0.0, 0.0), (2.0, 2.0, 2.0)).rotate_y(30.0).translate((5.0, 0.0, 0.0))
    centre = (5.0 + math.cos(math.radians(30)) * 1.0 + math.sin(math.radians(30)) * 1.0, 1.0,
              -math.sin(math.radians(30)) * 1.0 + math.cos(math.radians(30)) * 1.0)
    o = (centre[0], centre[1], centre[2] + 10.0)
    through = list(o) + [0.0, 0.0, -1.0]
    t, n = oracle.medium_hit(box, 1e9, through, 0.001, INF, 3)
    assert n == 1 and t is not None and 8.0 < t < 10.0
    t_thin, n = oracle.medium_hit(box, 1e-9, through, 0.001, INF, 3)
    assert n == 1 and t_thin is None
    t, n = oracle.medium_hit(box, 1.0, through, 0.001, 5.0, 3)
    assert n == 0 and t is None
    t, n = oracle.medium_hit(box, 1.0, list(o) + [0.0, 1.0, 0.0], 0.001, INF, 3)
    assert n == 0 and t is None
    # starting inside: the entry is behind the origin, clamped to tmin
    t, n = oracle.medium_hit(box, 1e9, list(centre) + [0.0, 0.0, 1.0], 0.001, INF, 9)
    assert n == 1 and t is not None and 0.001 <= t < 0.01
    # a box that is not translated or rotated is the same medium as one that is (0, +0)
    a = MediumBoundary.box((-1, -1, -1), (1, 1, 1))
    b = MediumBoundary.box((-1, -1, -1), (1, 1, 1)).rotate_y(0.0).translate((0.0, 0.0, 0.0))
    ray = [0.3, 0.2, 5.0, 0.01, -0.02, -1.0]
    assert oracle.medium_hit(a, 0.7, ray, 0.001, INF, 11) == oracle.medium_hit(b, 0.7, ray, 0.001, INF, 11)


def test_scene_media_validation():
    scene = RayScene()
    with pytest.raises(ValueError):
        scene.add_constant_medium(MediumBoundary.sphere((0, 0, 0), 1.0), 0.0, (1, 1, 1))
    with pytest.raises(ValueError):
        scene.add_constant_medium(MediumBoundary.sphere((0, 0, 0), 1.0), math.inf, (1, 1, 1))
    with pytest.raises(ValueError):
        MediumBoundary.box((0, 0, 0), (1, 1, 1)).translate((1, 0, 0)).rotate_y(10.0)
    k = scene.add_medium_with_phase_function(MediumBoundary.sphere((0, 0, 0), 1.0), 2.0,
                                             RayMaterial.henyey_greenstein((0.5, 0.5, 0.5), 0.3))
    assert k == 0 and scene.material_count() == 1


def test_smoke_scene_oracle_render():
    # cornell_smoke_world renders in the oracle in both precisions; the media change the
    # image against the same walls without them.
    scene, lights = scenes.cornell_smoke_scene()
    assert len(scene.media()) == 2
    cam = scenes.cornell_camera(24, 2, 8)
    o = oracle.OracleScene.from_ray_scene(scene)
    img, acc = o.render(cam.desc(), None, None, precision=1, threads=8)
    img32, _ = o.render(cam.desc(), None, None, precision=0, threads=8)
    assert np.isfinite(img).all() and np.isfinite(img32).all()
    bare = RayScene()
    for m in range(4):
        bare.add_material(scene._materials[m])
    bare.add_primitives_array(scene.primitives_array())
    bare.build_bvh()
    img_bare, _ = oracle.OracleScene.from_ray_scene(bare).render(cam.desc(), None, None, precision=1, threads=8)
    assert np.abs(img - img_bare).max() > 1e-3
