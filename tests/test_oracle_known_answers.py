"""Pins the CPU oracle to the reference's own known-answer tests.

Each test restates one assertion from the gartus test-suite (file:line given) and checks
the oracle against it.  These run without a GPU.
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from gartus_gb300 import abi, scenes
from gartus_gb300.raytracing import LIGHT_DTYPE, EnvironmentLight, RayCamera
from tests.helpers import dptr, geometry, material

L = oracle.lib()
INF = math.inf


def close(a, b, tol=1e-10):
    assert abs(a - b) < tol, (a, b)


def intersect(g, origin, direction, tmin=0.0, tmax=INF, time=0.0):
    out = (C.c_double * 10)()
    ok = L.orc_intersect(C.byref(g), dptr(list(origin) + list(direction) + [time]), tmin, tmax, out)
    return list(out) if ok else None


# ---------------------------------------------------------------- RNG / seeds
def test_splitmix64_known_stream():
    # SplitMix64 (the published generator SampleRng restates, gmath/random.rs:23-29):
    # seed 0 starts 0xe220a8397b1dcdaf, 0x6e789e6aa1b965f4, 0x06c45d188009454f.
    out = (C.c_uint64 * 3)()
    L.orc_rng_u64(0, 3, out)
    assert list(out) == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_random_double_half_open():  # gmath/random.rs:202-212
    out = (C.c_double * 200)()
    L.orc_rng_double(7, 200, out)
    assert all(0.0 <= v < 1.0 for v in out)


def test_python_generator_rng_matches_oracle():
    # The scene generators' SampleRng and the oracle's are the same stream.
    out = (C.c_uint64 * 16)()
    L.orc_rng_u64(61, 16, out)
    r = scenes.SampleRng(61)
    assert [r.next_u64() for _ in range(16)] == list(out)
    for (s, x, y) in [(1, 0, 0), (1, 399, 224), (0x5EED2026, 17, 3), (2**64 - 1, 5, 9)]:
        assert L.orc_pixel_seed(s, x, y) == scenes.pixel_seed(s, x, y)


# ------------------------------------------------------------ intersections
def test_sphere_roots():  # graphics/raytracing.rs:336-352
    s = geometry(abi.GT_GEOM_SPHERE, (0, 0, -1), 0.5)
    close(intersect(s, (0, 0, 0), (0, 0, -1))[0], 0.5)
    close(intersect(s, (0, 0, 0), (0, 0, -1), tmin=0.6)[0], 1.5)
    assert intersect(s, (0, 0, 0), (0, 1, -1)) is None
    assert intersect(s, (0, 0, 0), (0, 0, 0)) is None


def test_sphere_uv_reference_points():  # graphics/raytracing.rs:747-767 via hit u,v
    s = geometry(abi.GT_GEOM_SPHERE, (0, 0, 0), 1.0)
    cases = [((-3, 0, 0), (1, 0, 0), (0.0, 0.5)), ((3, 0, 0), (-1, 0, 0), (0.5, 0.5)),
             ((0, 3, 0), (0, -1, 0), (0.5, 1.0)), ((0, -3, 0), (0, 1, 0), (0.5, 0.0)),
             ((0, 0, 3), (0, 0, -1), (0.25, 0.5)), ((0, 0, -3), (0, 0, 1), (0.75, 0.5))]
    for o, d, (u, v) in cases:
        h = intersect(s, o, d)
        close(h[1], u)
        close(h[2], v)


def test_sphere_front_face_and_unit_normal():  # graphics/raytracing.rs:786-806
    s = geometry(abi.GT_GEOM_SPHERE, (0, 0, -1), 0.5)
    h = intersect(s, (0, 0, 0), (0, 0, -1))
    assert h[9] == 1.0
    assert h[6:9] == [0.0, 0.0, 1.0]


def test_triangle_barycentrics():  # gmath/geometry.rs:645-661
    t = geometry(abi.GT_GEOM_TRIANGLE, (0, 0, -1), (1, 0, -1), (0, 1, -1))
    h = intersect(t, (0.25, 0.25, 0), (0, 0, -1))
    close(h[0], 1.0)
    close(h[1], 0.25)
    close(h[2], 0.25)


def test_triangle_bounds_padding():  # gmath/geometry.rs:630-643
    t = geometry(abi.GT_GEOM_TRIANGLE, (0, 0, -1), (1, 0, -1), (0, 1, -1))
    b = (C.c_double * 6)()
    L.orc_geometry_bounds(C.byref(t), b)
    close(b[0], 0.0)
    close(b[2], -1.0 - 0.5e-10)
    close(b[5], -1.0 + 0.5e-10)


def test_triangle_rejects():  # graphics/raytracing.rs:1807-1833
    t = geometry(abi.GT_GEOM_TRIANGLE, (0, 0, -1), (1, 0, -1), (0, 1, -1))
    assert intersect(t, (1.1, 0.1, 0), (0, 0, -1)) is None
    assert intersect(t, (0.25, 0.25, -1), (1, 0, 0)) is None
    assert intersect(t, (0.25, 0.25, -2), (0, 0, -1)) is None
    deg = geometry(abi.GT_GEOM_TRIANGLE, (0, 0, -1), (0.5, 0, -1), (1, 0, -1))
    assert intersect(deg, (0.25, 0, 0), (0, 0, -1)) is None


def test_quad_planar_coordinates():  # gmath/geometry.rs:682-698, graphics/raytracing.rs:895-926
    q = geometry(abi.GT_GEOM_QUAD, (-2, -2, -1), (4, 0, 0), (0, 4, 0))
    h = intersect(q, (0, 1, 0), (0, 0, -1))
    close(h[0], 1.0)
    close(h[1], 0.5)
    close(h[2], 0.75)
    assert h[6:9] == [0.0, 0.0, 1.0] and h[9] == 1.0


def test_quad_rejects_and_bounds():  # gmath/geometry.rs:663-680, 700-726
    q = geometry(abi.GT_GEOM_QUAD, (-1, -1, -1), (2, 0, 0), (0, 2, 0))
    assert intersect(q, (2, 0, 0), (0, 0, -1)) is None
    assert intersect(q, (0, 0, 0), (1, 0, 0)) is None
    deg = geometry(abi.GT_GEOM_QUAD, (0, 0, 0), (1, 0, 0), (2, 0, 0))
    assert intersect(deg, (0, 0, 1), (0, 0, -1)) is None
    q2 = geometry(abi.GT_GEOM_QUAD, (-2, -2, 0), (4, 0, 0), (0, 4, 0))
    b = (C.c_double * 6)()
    L.orc_geometry_bounds(C.byref(q2), b)
    close(b[0], -2.0)
    close(b[4], 2.0)
    close(b[2], -0.5e-4)
    close(b[5], 0.5e-4)


# --------------------------------------------------------------------- PDFs
def test_quad_light_pdf():  # graphics/raytracing.rs:929-943
    q = geometry(abi.GT_GEOM_QUAD, (-1, -1, -1), (2, 0, 0), (0, 2, 0))
    close(L.orc_geometry_pdf(C.byref(q), dptr([0, 0, 0]), 0.0, dptr([0, 0, -1])), 0.25)
    close(L.orc_geometry_pdf(C.byref(q), dptr([0, 0, 0]), 0.0, dptr([0, 1, 0])), 0.0)


def test_sphere_light_pdf_is_inverse_solid_angle():  # graphics/raytracing.rs:946-964
    s = geometry(abi.GT_GEOM_SPHERE, (0, 0, -1), 0.5)
    solid = 2.0 * math.pi * (1.0 - math.sqrt(0.75))
    close(L.orc_geometry_pdf(C.byref(s), dptr([0, 0, 0]), 0.0, dptr([0, 0, -1])), 1.0 / solid)
    close(L.orc_geometry_pdf(C.byref(s), dptr([0, 0, 0]), 0.0, dptr([0, 1, 0])), 0.0)


def test_cosine_pdf_accepts_non_unit_directions():  # graphics/raytracing.rs:369-375
    close(L.orc_cosine_pdf(dptr([0, 1, 0]), dptr([0, 2, 0])), 1.0 / math.pi)
    close(L.orc_cosine_pdf(dptr([0, 1, 0]), dptr([0, 0, 0])), 0.0)
    close(L.orc_cosine_pdf(dptr([0, 1, 0]), dptr([0, -2, 0])), 0.0)


def test_weighted_target_selection_ratio():  # graphics/raytracing.rs:1658-1678
    # Two targets of weight 1 and 3: the heavier one is picked 75% +- 2.5% of the time.
    lights = np.zeros(2, dtype=LIGHT_DTYPE)
    lights[0]["geometry"]["kind"] = abi.GT_GEOM_QUAD
    lights[0]["geometry"]["p"][:9] = (-1, -1, -5, 2, 0, 0, 0, 2, 0)
    lights[0]["weight"] = 3.0
    lights[1]["geometry"]["kind"] = abi.GT_GEOM_QUAD
    lights[1]["geometry"]["p"][:9] = (-1, -1, 5, 2, 0, 0, 0, 2, 0)
    lights[1]["weight"] = 1.0
    frac = L.orc_lights_first_fraction(lights.ctypes.data_as(C.c_void_p), 2, dptr([0, 0, 0]), 149, 10000)
    assert abs(frac - 0.75) < 0.025


# ---------------------------------------------------------------- materials
def test_ggx_helpers():  # gmath/sampling.rs:518-536
    assert L.orc_ggx_d(1.0, 0.2) > L.orc_ggx_d(1.0, 0.8)
    close(L.orc_ggx_g(1.0, 1.0, 0.5), 1.0)
    close(L.orc_schlick(1.0, 0.04), 0.04)
    close(L.orc_schlick(0.0, 0.04), 1.0)


def test_dielectric_reflectance_grazing():  # graphics/raytracing.rs:1136-1142
    assert L.orc_dielectric_reflectance(0.1, 1.5) > L.orc_dielectric_reflectance(1.0, 1.5)


def _scatter(mat, ray, point, normal, front, seed):
    d = (C.c_double * 3)()
    a = (C.c_double * 3)()
    st = C.c_uint64()
    k = L.orc_scatter(C.byref(mat), dptr(ray), dptr(point), dptr(normal), int(front), seed, d, a, C.byref(st))
    return k, list(d), list(a)


def test_dielectric_refracts_perpendicular_ray():  # graphics/raytracing.rs:1108-1134
    m = material(abi.GT_MAT_DIELECTRIC, (1, 1, 1), 1.5)
    k, d, a = _scatter(m, [0, 0, 0, 0, 0, -1, 0.625], [0, 0, -0.5], [0, 0, 1], True, 23)
    assert k == 1 and d == [0.0, 0.0, -1.0] and a == [1.0, 1.0, 1.0]


def test_metal_mirror_reflection():  # graphics/raytracing.rs:1080-1106 (fuzz 0)
    m = material(abi.GT_MAT_METAL, (0.8, 0.8, 0.8), 0.0)
    k, d, a = _scatter(m, [0, 0, 0, 0, 0, -1, 0.0], [0, 0, -0.5], [0, 0, 1], True, 19)
    assert k == 1
    assert d[0] == 0.0 and d[1] == 0.0 and d[2] == 1.0
    assert a == [0.8, 0.8, 0.8]


def test_metal_fuzz_clamp():  # graphics/raytracing.rs:770-784
    m = material(abi.GT_MAT_METAL, (0.8, 0.6, 0.2), 2.0)  # clamped to 1 at load
    k, d, a = _scatter(m, [0, 0, 0, 0, 0, -1, 0.0], [0, 0, -0.5], [0, 0, 1], True, 5)
    assert k in (0, 1)
    if k == 1:
        assert math.sqrt(sum((x - y) ** 2 for x, y in zip(d, (0, 0, 1)))) <= 1.0 + 1e-12


def test_lambertian_scattering_pdf():  # material.rs:523-530
    m = material(abi.GT_MAT_LAMBERTIAN, (0.2, 0.4, 0.6))
    close(L.orc_scattering_pdf(C.byref(m), dptr([0, 0, 0, 0, 0, -1, 0]), dptr([0, 0, -1]), dptr([0, 0, 1]), 1,
                               dptr([0, 0, 3])), 1.0 / math.pi)
    close(L.orc_scattering_pdf(C.byref(m), dptr([0, 0, 0, 0, 0, -1, 0]), dptr([0, 0, -1]), dptr([0, 0, 1]), 1,
                               dptr([0, 0, -3])), 0.0)


# --------------------------------------------------------------- integrator
def test_power_heuristic():  # camera.rs:2486-2496
    close(L.orc_power_heuristic(1.0, 1.0), 0.5)
    close(L.orc_power_heuristic(0.0, 1.0), 0.0)
    close(L.orc_power_heuristic(2.0, 0.0), 1.0)


def test_adaptive_error():  # graphics/camera.rs:4967-4973
    m2 = dptr([1.0, 4.0, 9.0])
    close(L.orc_adaptive_error(m2, 4), math.sqrt(0.75))
    assert math.isinf(L.orc_adaptive_error(m2, 1))


def test_sky_gradient():  # graphics/raytracing.rs:355-366 (sky_gradient as a RayBackground)
    cam = scenes.final_scene_camera(40, 1).desc()
    out = (C.c_double * 3)()
    L.orc_background(C.byref(cam), dptr([0, 0, -1]), out)
    close(out[0], 0.75)
    close(out[1], 0.85)
    close(out[2], 1.0)


def test_environment_pdf_half_sphere():  # raytracing/environment.rs:249-269
    env = EnvironmentLight(np.array([[[255, 255, 255]], [[0, 0, 0]]], dtype=np.uint8))
    close(L.orc_env_pdf(C.byref(env.desc()), dptr([0, 1, 0])), 1.0 / (2.0 * math.pi), 1e-12)
    close(L.orc_env_pdf(C.byref(env.desc()), dptr([1, 0.5, 0])), 1.0 / (2.0 * math.pi), 1e-12)


def _empty_scene():
    from gartus_gb300.raytracing import RayScene, RayMaterial
    s = RayScene()
    s.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    return s


def test_hdr_passthrough_and_adaptive_min_samples():  # graphics/camera.rs:4975-5004
    # A miss-only world: the pixel is exactly the background, above display white, and
    # zero variance stops adaptive sampling at its minimum.
    s = oracle.OracleScene.from_ray_scene(_empty_scene())
    cam = RayCamera(1, 1.0).with_background((4.0, 2.0, 0.25)).with_samples_per_pixel(1)
    rgb, acc = s.render(cam.desc())
    assert list(rgb[0, 0]) == [4.0, 2.0, 0.25] and acc[0, 0] == 1
    cam = RayCamera(1, 1.0).with_background((0.25, 0.25, 0.25)).with_adaptive_sampling(4, 16, 0.001)
    rgb, acc = s.render(cam.desc())
    assert acc[0, 0] == 4 and list(rgb[0, 0]) == [0.25, 0.25, 0.25]


# --------------------------------------------------------------------- BVH
def test_bvh_matches_bruteforce_randomized():  # graphics/raytracing.rs:1340-1370
    for seed in range(1, 17):
        scene = scenes.randomized_ray_scene(seed)
        o = oracle.OracleScene.from_ray_scene(scene)
        rr = scenes.SampleRng(seed ^ 0x9E3779B97F4A7C15)
        rays = np.zeros((64, 7))
        for i in range(64):
            org = (rr.random_range(-4.0, 4.0), rr.random_range(-3.0, 3.0), rr.random_range(0.0, 3.0))
            tgt = (rr.random_range(-3.0, 3.0), rr.random_range(-2.0, 2.0), rr.random_range(-8.0, -1.0))
            rays[i, :3] = org
            rays[i, 3:6] = (tgt[0] - org[0], tgt[1] - org[1], tgt[2] - org[2])
        ib, tb, hb, _ = o.trace(rays)
        ibf, tbf, hbf, _ = o.trace(rays, bruteforce=True)
        assert (ib >= 0).sum() > 0
        np.testing.assert_array_equal(ib >= 0, ibf >= 0)
        hit = ib >= 0
        np.testing.assert_allclose(tb[hit], tbf[hit], atol=1e-10)
        np.testing.assert_allclose(hb[hit, :6], hbf[hit, :6], atol=1e-10)


def test_bvh_leaf_size_controls_node_count():  # graphics/raytracing.rs:1884-1905
    tris = []
    for i in range(8):
        x = float(i)
        tris.append([(x, 0.0, -1.0), (x + 0.5, 0.0, -1.0), (x, 0.5, -1.0)])
    from gartus_gb300.raytracing import RayScene, RayMaterial
    small, large = RayScene(), RayScene()
    for s, leaf in ((small, 1), (large, 8)):
        m = s.add_material(RayMaterial.lambertian((0.2, 0.2, 0.2)))
        s.add_triangles_array(m, np.array(tris))
        s.build_bvh_with_options(leaf)
    n_small = oracle.OracleScene.from_ray_scene(small).node_count()
    n_large = oracle.OracleScene.from_ray_scene(large).node_count()
    assert n_small > n_large and n_large == 1


def test_final_scene_shape():  # raytracing/scenes.rs:563-624
    s = scenes.final_scene_ray_scene()
    kinds = s.materials_array()["kind"]
    assert len(s) == s.material_count()
    assert 450 <= len(s) <= 488
    # Ground, then the three big spheres last.
    p = s.primitives_array()
    assert tuple(p[0]["geometry"]["p"][:4]) == (0.0, -1000.0, 0.0, 1000.0)
    assert tuple(p[-1]["geometry"]["p"][:4]) == (4.0, 1.0, 0.0, 1.0)
    assert kinds[-1] == abi.GT_MAT_METAL and kinds[-3] == abi.GT_MAT_DIELECTRIC


def test_oracle_render_deterministic_and_finite():  # graphics/camera.rs:5317-5330
    s = scenes.final_scene_ray_scene()
    o = oracle.OracleScene.from_ray_scene(s)
    cam = scenes.final_scene_camera(32, 2).desc()
    a, acc_a = o.render(cam, threads=4)
    b, acc_b = o.render(cam, threads=1)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(acc_a, acc_b)
    assert np.isfinite(a).all() and a.mean() > 0.05


def test_oracle_window_matches_full_image():
    s = scenes.final_scene_ray_scene()
    o = oracle.OracleScene.from_ray_scene(s)
    cam = scenes.final_scene_camera(32, 2).desc()
    full, _ = o.render(cam, threads=4)
    part, _ = o.render(cam, threads=2, window=(5, 3, 9, 7))
    np.testing.assert_array_equal(full[3:10, 5:14], part)


# ---------------------------------------------------------------- Perlin noise
def _perlin(seed, pts, depth=-1, precision=1):
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros(len(pts))
    oracle.lib().orc_perlin(seed, precision, depth, len(pts), pts.ctypes.data, out.ctypes.data)
    return out


def _perlin_python(seed, p):
    """A second, independent restatement of Perlin::new + Perlin::noise (gmath/perlin.rs:19-58,
    83-136) in plain Python floats, to pin the oracle's C++ version."""
    state = seed

    def unit():
        nonlocal state
        state = (state + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        v = state
        v = ((v ^ (v >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        v = ((v ^ (v >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return ((v ^ (v >> 31)) >> 11) * (1.0 / 9007199254740992.0)

    grads = []
    for _ in range(256):
        r1, r2 = unit(), unit()
        z = 1.0 - 2.0 * r2
        radius = math.sqrt(1.0 - z * z)
        phi = 6.283185307179586 * r1
        grads.append((math.cos(phi) * radius, math.sin(phi) * radius, z))
    perms = []
    for _ in range(3):
        q = list(range(256))
        for i in range(255, 0, -1):
            t = int(unit() * (i + 1.0))
            q[i], q[t] = q[t], q[i]
        perms.append(q)
    fx, fy, fz = (c - math.floor(c) for c in p)
    bx, by, bz = (int(math.floor(c)) for c in p)
    s = [v * v * (3.0 - 2.0 * v) for v in (fx, fy, fz)]
    acc = 0.0
    for ox in (0, 1):
        for oy in (0, 1):
            for oz in (0, 1):
                g = grads[perms[0][(bx + ox) & 255] ^ perms[1][(by + oy) & 255] ^ perms[2][(bz + oz) & 255]]
                dot = g[0] * (fx - ox) + g[1] * (fy - oy) + g[2] * (fz - oz)
                bw = (s[0] if ox else 1.0 - s[0]) * (s[1] if oy else 1.0 - s[1]) * (s[2] if oz else 1.0 - s[2])
                acc += bw * dot
    return acc


def test_perlin_repeatable_for_same_seed():  # gmath/perlin.rs:152-161
    p = [[1.25, -0.5, 3.75]]
    assert _perlin(7, p)[0] == _perlin(7, p)[0]
    assert _perlin(7, p, depth=7)[0] == _perlin(7, p, depth=7)[0]


def test_perlin_varies_with_seed_and_position():  # gmath/perlin.rs:163-173
    a = _perlin(7, [[1.25, -0.5, 3.75], [1.5, -0.5, 3.75]])
    b = _perlin(8, [[1.25, -0.5, 3.75]])
    assert abs(a[0] - b[0]) > 2.220446049250313e-16
    assert abs(a[0] - a[1]) > 2.220446049250313e-16


def test_perlin_turbulence_non_negative():  # gmath/perlin.rs:175-180
    assert _perlin(11, [[0.2, 0.4, 0.6]], depth=7)[0] >= 0.0


def test_perlin_matches_independent_restatement():
    rng = np.random.default_rng(5)
    pts = rng.uniform(-40.0, 40.0, size=(24, 3))
    pts[0] = (0.0, 0.0, 0.0)     # lattice point: noise 0
    pts[1] = (-0.5, 255.5, 256.25)  # wraps the 256-entry tables
    for seed in (1, 7, 1 << 40):
        got = _perlin(seed, pts)
        want = [_perlin_python(seed, p) for p in pts]
        np.testing.assert_array_equal(got, want)
    assert _perlin(3, [[0.0, 0.0, 0.0]])[0] == 0.0
    # turbulence = |sum_k 0.5^k noise(2^k p)|
    p = pts[2]
    want = abs(sum(0.5 ** k * _perlin(9, [p * 2.0 ** k])[0] for k in range(5)))
    assert abs(_perlin(9, [p], depth=5)[0] - want) <= 1e-15


def _hg_pdf(g, forward, direction):
    m = material(abi.GT_MAT_HENYEY_GREENSTEIN, (0.5, 0.5, 0.5), g)
    return L.orc_scattering_pdf(C.byref(m), dptr([0, 0, 0] + list(forward) + [0]), dptr([0, 0, 0]),
                                dptr([0, 0, 1]), 1, dptr(direction))


def test_henyey_greenstein_pdf_biases_forward_or_backward():  # gmath/sampling.rs:485-497
    close(_hg_pdf(0.0, (0, 0, 1), (0.25, 0.0, math.sqrt(1 - 0.0625))), 1.0 / (4.0 * math.pi))
    assert _hg_pdf(0.6, (0, 0, 1), (0, 0, 1)) > _hg_pdf(0.6, (0, 0, 1), (0, 0, -1))
    assert _hg_pdf(-0.6, (0, 0, 1), (0, 0, -1)) > _hg_pdf(-0.6, (0, 0, 1), (0, 0, 1))
    # the phase function of g: (1 - g^2) / (4 pi (1 + g^2 - 2 g cos)^1.5), and 0 for a null direction
    g, c = 0.3, 0.5
    close(_hg_pdf(g, (0, 0, 2), (math.sqrt(1 - c * c), 0, c)),
          (1 - g * g) / (4 * math.pi * (1 + g * g - 2 * g * c) ** 1.5))
    assert _hg_pdf(g, (0, 0, 1), (0, 0, 0)) == 0.0


def test_henyey_greenstein_samples_mean_cosine_near_anisotropy():  # gmath/sampling.rs:499-514
    g = 0.55
    m = material(abi.GT_MAT_HENYEY_GREENSTEIN, (0.2, 0.4, 0.6), g)
    total = 0.0
    n = 8192
    for seed in range(n):
        k, d, a = _scatter(m, [0, 0, 0, 0, 0, 3, 0], [0, 0, 0], [0, 0, 1], True, 107 + seed)
        assert k == 2 and a == [0.2, 0.4, 0.6]  # a pdf scatter with the albedo
        assert abs(math.sqrt(sum(x * x for x in d)) - 1.0) <= 1e-12
        total += d[2]
    assert abs(total / n - g) <= 0.035


def test_decision_trace_adaptive_stop_and_substreams():
    # The decision trace records each adaptive stop test (type 14: outcome 1 = stop, value
    # (error - threshold) / threshold); the pixel's accepted samples end at the first stop.
    # With per-sample substreams the same pixel takes other decisions (its own streams).
    scene, lights = scenes.batch_scene()
    cam = scenes.batch_cameras(frames=3, width=24, spp_cycle=(4,), max_samples=64, threshold=0.05)[1]
    o = oracle.OracleScene.from_ray_scene(scene)
    la = lights.to_array()
    rgb, acc = o.render(cam.desc(), la, None, precision=1, threads=4)
    y, x = 12, 12
    types, outcomes, values = o.pixel_trace(cam.desc(), x, y, la, None, precision=1)
    adaptive = np.flatnonzero(types == 14)
    assert adaptive.size > 0
    stops = np.flatnonzero((types == 14) & (outcomes == 1))
    # every test before the stop continued, with the error above the threshold
    assert np.all(values[adaptive[outcomes[adaptive] == 0]] >= 0)
    if stops.size:
        assert stops[0] == adaptive[-1] and values[stops[0]] < 0
    samples = np.count_nonzero((types == 1) & (outcomes == 1))
    assert samples == acc[y, x]
    t_sub = o.pixel_trace(cam.desc(), x, y, la, None, precision=1, rng="substreams")
    assert not (len(t_sub[0]) == len(types) and np.array_equal(t_sub[1], outcomes) and np.array_equal(t_sub[2], values))
    sub, _ = o.render(cam.desc(), la, None, precision=1, threads=4, rng="substreams")
    assert sub.shape == rgb.shape and not np.array_equal(sub, rgb)
