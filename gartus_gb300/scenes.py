"""Seeded scene generators: the reference's own scenes and the synthetic workloads built
from them (raytracing/scenes.rs, benches/render_performance.rs, raytracing.rs tests).

Python floats are IEEE f64 without fused multiply-add, and math.sin/cos/sqrt call the C
library, so the geometry below is bit-identical to what the Rust generators produce.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from .raytracing import GLASS, MediumBoundary, RayCamera, RayMaterial, RayScene, SamplingTargetList

MASK = 0xFFFFFFFFFFFFFFFF


class SampleRng:
    """SampleRng (gmath/random.rs:16-153): SplitMix64."""

    def __init__(self, seed: int):
        self.state = seed & MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK
        v = self.state
        v = ((v ^ (v >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        v = ((v ^ (v >> 27)) * 0x94D049BB133111EB) & MASK
        return v ^ (v >> 31)

    def random_double(self) -> float:
        return float(self.next_u64() >> 11) * (1.0 / 9007199254740992.0)

    def random_range(self, lo: float, hi: float) -> float:
        return lo + (hi - lo) * self.random_double()

    def random_vector(self) -> tuple:
        a = self.random_double()
        b = self.random_double()
        c = self.random_double()
        return (a, b, c)

    def random_vector_range(self, lo, hi) -> tuple:
        a = self.random_range(lo, hi)
        b = self.random_range(lo, hi)
        c = self.random_range(lo, hi)
        return (a, b, c)

    def random_unit_vector(self) -> tuple:  # random.rs:107-115
        r1 = self.random_double()
        r2 = self.random_double()
        z = 1.0 - 2.0 * r2
        radius = math.sqrt(1.0 - z * z)
        phi = 6.283185307179586 * r1
        return (math.cos(phi) * radius, math.sin(phi) * radius, z)


def pixel_seed(seed: int, x: int, y: int) -> int:
    """RayCamera::pixel_seed (graphics/camera.rs:1720-1727)."""
    z = (seed ^ ((x * 0x9E3779B97F4A7C15) & MASK) ^ ((y * 0xD1B54A32D192ED03) & MASK)) & MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    return z ^ (z >> 31)


# ----------------------------------------------------------- final scene (cfg 0)
def final_scene_ray_scene() -> RayScene:
    """final_scene_ray_scene (raytracing/scenes.rs:563-624), seed 61: ground sphere, a
    22x22 grid of small spheres (80% Lambertian, 15% Metal, 5% Dielectric) and three
    large spheres."""
    rng = SampleRng(61)
    world = RayScene()
    world.add_sphere_with_material((0.0, -1000.0, 0.0), 1000.0, RayMaterial.lambertian((0.5, 0.5, 0.5)))
    for a in range(-11, 11):
        for b in range(-11, 11):
            choose = rng.random_double()
            cx = float(a) + 0.9 * rng.random_double()
            cz = float(b) + 0.9 * rng.random_double()
            center = (cx, 0.2, cz)
            d = (cx - 4.0, 0.2 - 0.2, cz - 0.0)
            if math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) <= 0.9:
                continue
            if choose < 0.8:
                v1 = rng.random_vector()
                v2 = rng.random_vector()
                albedo = (v1[0] * v2[0], v1[1] * v2[1], v1[2] * v2[2])
                world.add_sphere_with_material(center, 0.2, RayMaterial.lambertian(albedo))
            elif choose < 0.95:
                albedo = rng.random_vector_range(0.5, 1.0)
                fuzz = rng.random_range(0.0, 0.5)
                world.add_sphere_with_material(center, 0.2, RayMaterial.metal(albedo, fuzz))
            else:
                world.add_sphere_with_material(center, 0.2, RayMaterial.dielectric(GLASS))
    world.add_sphere_with_material((0.0, 1.0, 0.0), 1.0, RayMaterial.dielectric(GLASS))
    world.add_sphere_with_material((-4.0, 1.0, 0.0), 1.0, RayMaterial.lambertian((0.4, 0.2, 0.1)))
    world.add_sphere_with_material((4.0, 1.0, 0.0), 1.0, RayMaterial.metal((0.7, 0.6, 0.5), 0.0))
    world.build_bvh()
    return world


def final_scene_camera(width: int = 400, spp: int = 32) -> RayCamera:
    """The book's final-scene camera (examples/raytracing/weekend.rs:116-130) with the
    vertical sky gradient of scenes.rs:17-21 as a RayBackground."""
    return (RayCamera(width, 16.0 / 9.0)
            .with_samples_per_pixel(spp)
            .with_max_depth(10)
            .with_vertical_fov(20.0)
            .with_look_at((13.0, 2.0, 3.0), (0.0, 0.0, 0.0))
            .with_view_up((0.0, 1.0, 0.0))
            .with_defocus_angle(0.6)
            .with_focus_distance(10.0)
            .with_vertical_gradient_background((1.0, 1.0, 1.0), (0.75, 0.85, 1.0), (0.5, 0.7, 1.0)))


# ---------------------------------------------------------------- Cornell (cfg 1)
def _rotate_y(v, s, c):  # rotate_y_vector, raytracing/instance.rs:395-401
    return (c * v[0] + s * v[2], v[1], -s * v[0] + c * v[2])


def _box_quads(a, b):
    """box_object (raytracing/object.rs:930-976): six quads of an axis-aligned box."""
    mn = (min(a[0], b[0]), min(a[1], b[1]), min(a[2], b[2]))
    mx = (max(a[0], b[0]), max(a[1], b[1]), max(a[2], b[2]))
    dx = (mx[0] - mn[0], 0.0, 0.0)
    dy = (0.0, mx[1] - mn[1], 0.0)
    dz = (0.0, 0.0, mx[2] - mn[2])
    neg = lambda v: (-v[0], -v[1], -v[2])  # noqa: E731
    return [
        ((mn[0], mn[1], mx[2]), dx, dy),
        ((mx[0], mn[1], mx[2]), neg(dz), dy),
        ((mx[0], mn[1], mn[2]), neg(dx), dy),
        ((mn[0], mn[1], mn[2]), dz, dy),
        ((mn[0], mx[1], mx[2]), dx, neg(dz)),
        ((mn[0], mn[1], mn[2]), dx, dz),
    ]


def rotated_box_quads(a, b, angle_degrees, offset):
    """A box under Translate(RotateY(box, angle), offset) flattened to world-space quads:
    corners rotated then translated, edge vectors rotated (instance.rs:96-202, 379-401)."""
    rad = angle_degrees * math.pi / 180.0  # degrees_to_radians, raytracing.rs:150-152
    s, c = math.sin(rad), math.cos(rad)
    out = []
    for corner, u, v in _box_quads(a, b):
        rc = _rotate_y(corner, s, c)
        out.append(((rc[0] + offset[0], rc[1] + offset[1], rc[2] + offset[2]), _rotate_y(u, s, c), _rotate_y(v, s, c)))
    return out


def cornell_scene() -> tuple[RayScene, SamplingTargetList]:
    """The Cornell box of cornell_box_world (raytracing/scenes.rs:226-294) as a RayScene:
    five walls and the ceiling light, the tall 165x330x165 box rotated 15 degrees as a
    GGX microfacet (base colour 0.8, roughness 0.3) and a Dielectric(1.5) sphere of radius
    90 in place of the short box.  The light quad is the only sampling target."""
    scene = RayScene()
    red = scene.add_material(RayMaterial.lambertian((0.65, 0.05, 0.05)))
    white = scene.add_material(RayMaterial.lambertian((0.73, 0.73, 0.73)))
    green = scene.add_material(RayMaterial.lambertian((0.12, 0.45, 0.15)))
    light = scene.add_material(RayMaterial.diffuse_light((15.0, 15.0, 15.0)))
    ggx = scene.add_material(RayMaterial.ggx_microfacet((0.8, 0.8, 0.8), 0.3))
    glass = scene.add_material(RayMaterial.dielectric(GLASS))
    scene.add_quad((555.0, 0.0, 0.0), (0.0, 555.0, 0.0), (0.0, 0.0, 555.0), green)
    scene.add_quad((0.0, 0.0, 0.0), (0.0, 555.0, 0.0), (0.0, 0.0, 555.0), red)
    scene.add_quad((343.0, 554.0, 332.0), (-130.0, 0.0, 0.0), (0.0, 0.0, -105.0), light)
    scene.add_quad((0.0, 0.0, 0.0), (555.0, 0.0, 0.0), (0.0, 0.0, 555.0), white)
    scene.add_quad((555.0, 555.0, 555.0), (-555.0, 0.0, 0.0), (0.0, 0.0, -555.0), white)
    scene.add_quad((0.0, 0.0, 555.0), (555.0, 0.0, 0.0), (0.0, 555.0, 0.0), white)
    for corner, u, v in rotated_box_quads((0.0, 0.0, 0.0), (165.0, 330.0, 165.0), 15.0, (265.0, 0.0, 295.0)):
        scene.add_quad(corner, u, v, ggx)
    scene.add_sphere((190.0, 90.0, 190.0), 90.0, glass)
    scene.build_bvh()
    lights = SamplingTargetList()
    lights.add_quad((343.0, 554.0, 332.0), (-130.0, 0.0, 0.0), (0.0, 0.0, -105.0))
    return scene, lights


def cornell_camera(width: int = 600, grid: int = 16, max_depth: int = 50) -> RayCamera:
    """examples/raytracing/next_weekend.rs:132-146 with a 16x16 stratified grid."""
    return (RayCamera(width, 1.0)
            .with_stratified_grid_width(grid)
            .with_max_depth(max_depth)
            .with_background((0.0, 0.0, 0.0))
            .with_vertical_fov(40.0)
            .with_look_at((278.0, 278.0, -800.0), (278.0, 278.0, 0.0))
            .with_view_up((0.0, 1.0, 0.0)))


def cornell_smoke_scene() -> tuple[RayScene, SamplingTargetList]:
    """cornell_smoke_world (raytracing/scenes.rs:296-378): the five walls and a 330x305
    ceiling light of radiance 7, and the two boxes of the Cornell box as constant-density
    media (density 0.01; black smoke in the tall box rotated 15 degrees, white smoke in the
    short one rotated -18 degrees), tested after the walls in that order.  The light quad
    is returned as a sampling target for next-event estimation."""
    scene = RayScene()
    red = scene.add_material(RayMaterial.lambertian((0.65, 0.05, 0.05)))
    white = scene.add_material(RayMaterial.lambertian((0.73, 0.73, 0.73)))
    green = scene.add_material(RayMaterial.lambertian((0.12, 0.45, 0.15)))
    light = scene.add_material(RayMaterial.diffuse_light((7.0, 7.0, 7.0)))
    scene.add_quad((555.0, 0.0, 0.0), (0.0, 555.0, 0.0), (0.0, 0.0, 555.0), green)
    scene.add_quad((0.0, 0.0, 0.0), (0.0, 555.0, 0.0), (0.0, 0.0, 555.0), red)
    scene.add_quad((113.0, 554.0, 127.0), (330.0, 0.0, 0.0), (0.0, 0.0, 305.0), light)
    scene.add_quad((0.0, 555.0, 0.0), (555.0, 0.0, 0.0), (0.0, 0.0, 555.0), white)
    scene.add_quad((0.0, 0.0, 0.0), (555.0, 0.0, 0.0), (0.0, 0.0, 555.0), white)
    scene.add_quad((0.0, 0.0, 555.0), (555.0, 0.0, 0.0), (0.0, 555.0, 0.0), white)
    tall = MediumBoundary.box((0.0, 0.0, 0.0), (165.0, 330.0, 165.0)).rotate_y(15.0).translate((265.0, 0.0, 295.0))
    short = MediumBoundary.box((0.0, 0.0, 0.0), (165.0, 165.0, 165.0)).rotate_y(-18.0).translate((130.0, 0.0, 65.0))
    scene.add_constant_medium(tall, 0.01, (0.0, 0.0, 0.0))
    scene.add_constant_medium(short, 0.01, (1.0, 1.0, 1.0))
    scene.build_bvh()
    lights = SamplingTargetList()
    lights.add_quad((113.0, 554.0, 127.0), (330.0, 0.0, 0.0), (0.0, 0.0, 305.0))
    return scene, lights


# -------------------------------------------------------- reference bench scene
def render_performance_scene() -> RayScene:
    """build_benchmark_scene (benches/render_performance.rs:10-29): 129 spheres."""
    scene = RayScene()
    ground = scene.add_material(RayMaterial.lambertian((0.45, 0.47, 0.43)))
    warm = scene.add_material(RayMaterial.lambertian((0.75, 0.45, 0.32)))
    cool = scene.add_material(RayMaterial.lambertian((0.25, 0.45, 0.78)))
    scene.add_sphere((0.0, -1000.65, -4.0), 1000.0, ground)
    for row in range(8):
        for column in range(16):
            x = (float(column) - 7.5) * 0.45
            z = -1.4 - float(row) * 0.55
            y = -0.35 + 0.04 * float((row + column) % 3)
            scene.add_sphere((x, y, z), 0.16, warm if (row + column) % 2 == 0 else cool)
    scene.build_bvh_with_options(4)
    return scene


def render_performance_camera() -> RayCamera:
    """benchmark_camera (benches/render_performance.rs:31-39)."""
    return (RayCamera(96, 16.0 / 9.0)
            .with_samples_per_pixel(2)
            .with_max_depth(5)
            .with_vertical_fov(35.0)
            .with_look_at((0.0, 1.1, 2.6), (0.0, -0.25, -3.4))
            .with_view_up((0.0, 1.0, 0.0))
            .with_rng_seed(0x5EED_2026))


# ----------------------------------------------------- randomized test scene
def randomized_ray_scene(seed: int) -> RayScene:
    """randomized_ray_scene (graphics/raytracing.rs:242-289): 8 spheres, 4 quads and
    4 triangles from one SampleRng stream."""
    rng = SampleRng(seed)
    scene = RayScene()
    m = scene.add_material(RayMaterial.lambertian((0.4, 0.5, 0.6)))
    for _ in range(8):
        c = (rng.random_range(-3.0, 3.0), rng.random_range(-2.0, 2.0), rng.random_range(-8.0, -1.0))
        r = rng.random_range(0.1, 0.45)
        scene.add_sphere(c, r, m)
    for _ in range(4):
        c = (rng.random_range(-3.0, 3.0), rng.random_range(-2.0, 2.0), rng.random_range(-8.0, -1.0))
        half = rng.random_range(0.15, 0.5)
        scene.add_quad((c[0] + -half, c[1] + -half, c[2] + 0.0), (2.0 * half, 0.0, 0.0), (0.0, 2.0 * half, 0.0), m)
    for _ in range(4):
        c = (rng.random_range(-3.0, 3.0), rng.random_range(-2.0, 2.0), rng.random_range(-8.0, -1.0))
        s = rng.random_range(0.2, 0.7)
        p0 = (c[0] + -s, c[1] + -s, c[2] + 0.0)
        p1 = (c[0] + s, c[1] + -s, c[2] + 0.0)
        dz = rng.random_range(-0.2, 0.2)
        p2 = (c[0] + 0.0, c[1] + s, c[2] + dz)
        scene.add_triangle(p0, p1, p2, m)
    scene.build_bvh()
    return scene


def random_rays(seed: int, count: int, origin_box=(-4.0, 4.0), z=(0.5, 2.0)) -> np.ndarray:
    """Seeded probe rays {origin, direction, time=0} aimed into -z (for hit tests)."""
    rng = SampleRng(seed)
    rays = np.zeros((count, 7), dtype=np.float64)
    for i in range(count):
        o = (rng.random_range(*origin_box), rng.random_range(-3.0, 3.0), rng.random_range(*z))
        t = (rng.random_range(-3.0, 3.0), rng.random_range(-2.0, 2.0), rng.random_range(-8.0, -1.0))
        rays[i, :3] = o
        rays[i, 3:6] = (t[0] - o[0], t[1] - o[1], t[2] - o[2])
    return rays


CONFIGS = {
    "final_scene": "400x225, 32 spp, depth 10, 486-sphere final scene (reference scenes.rs:563-624)",
    "cornell": "600x600, 16x16 stratified (256 spp), depth 50, GGX box + glass sphere, light-target mixture",
}


# ------------------------------------------------------- mesh-heavy scene (cfg 2)
def perlin_tables(seed: int) -> tuple[np.ndarray, np.ndarray]:
    """Perlin::new(seed) (gmath/perlin.rs:19-31, 83-101): 256 unit gradients, then the
    x, y, z permutations (identity shuffled from the last index down)."""
    rng = SampleRng(seed)
    grad = np.array([rng.random_unit_vector() for _ in range(256)], dtype=np.float64)
    perm = np.zeros((3, 256), dtype=np.int64)
    for axis in range(3):
        p = list(range(256))
        for i in range(255, 0, -1):
            t = int(rng.random_double() * (float(i) + 1.0))
            p[i], p[t] = p[t], p[i]
        perm[axis] = p
    return grad, perm


def perlin_noise(grad: np.ndarray, perm: np.ndarray, pts: np.ndarray) -> np.ndarray:
    """Perlin::noise (perlin.rs:36-58) with perlin_interp (106-124) over an (N, 3) array of
    points: the same f64 operations, in the same order, elementwise."""
    pts = np.asarray(pts, dtype=np.float64)
    fl = np.floor(pts)
    f = pts - fl
    base = fl.astype(np.int64)
    s = f * f * (3.0 - 2.0 * f)
    acc = np.zeros(len(pts))
    for ox in (0, 1):
        for oy in (0, 1):
            for oz in (0, 1):
                gi = (perm[0][(base[:, 0] + ox) & 255] ^ perm[1][(base[:, 1] + oy) & 255]
                      ^ perm[2][(base[:, 2] + oz) & 255])
                g = grad[gi]
                dot = g[:, 0] * (f[:, 0] - ox) + g[:, 1] * (f[:, 1] - oy) + g[:, 2] * (f[:, 2] - oz)
                bw = ((s[:, 0] if ox else 1.0 - s[:, 0]) * (s[:, 1] if oy else 1.0 - s[:, 1])
                      * (s[:, 2] if oz else 1.0 - s[:, 2]))
                acc = acc + bw * dot
    return acc


def height_map_triangles(heights: np.ndarray, x_size: float, z_size: float, height_scale: float,
                         y_offset: float = 0.0) -> np.ndarray:
    """PolygonMatrix::from_height_map (gmath/polygon_matrix.rs:510-541) as an (N, 3, 3)
    vertex array: per cell (row-major, z outer) the triangles (p00, p01, p11), (p00, p11, p10)."""
    rows, cols = heights.shape
    xs = (np.arange(cols, dtype=np.float64) / float(cols - 1) - 0.5) * x_size
    zs = (np.arange(rows, dtype=np.float64) / float(rows - 1) - 0.5) * z_size
    ys = heights * height_scale + y_offset
    X = np.broadcast_to(xs[None, :], (rows, cols))
    Z = np.broadcast_to(zs[:, None], (rows, cols))
    P = np.stack([X, ys, Z], axis=-1)
    p00, p10, p01, p11 = P[:-1, :-1], P[:-1, 1:], P[1:, :-1], P[1:, 1:]
    t0 = np.stack([p00, p01, p11], axis=2)
    t1 = np.stack([p00, p11, p10], axis=2)
    return np.stack([t0, t1], axis=2).reshape(-1, 3, 3)


def torus_triangles(center, radius_small: float, radius_big: float, rings: int, tube: int) -> np.ndarray:
    """PolygonMatrix::add_torus (gmath/polygon_matrix.rs:795-864) with separate ring and
    tube counts (the reference takes one `steps` for both): ring i, tube j gives the
    outward triangles (p0, p3, p2), (p0, p2, p1)."""
    cx, cy, cz = center
    theta = np.array([j * (1.0 / tube) * math.pi * 2.0 for j in range(tube)])
    sin_t, cos_t = np.sin(theta), np.cos(theta)
    ringpts = []
    for i in range(rings):
        phi = i * (1.0 / rings) * math.pi * 2.0
        sp, cp = math.sin(phi), math.cos(phi)
        x = cp * (radius_small * cos_t + radius_big) + cx
        y = radius_small * sin_t + cy
        z = -sp * (radius_small * cos_t + radius_big) + cz
        ringpts.append(np.stack([x, y, z], axis=-1))
    tris = []
    for i in range(rings):
        cur, nxt = ringpts[i], ringpts[(i + 1) % rings]
        j1 = (np.arange(tube) + 1) % tube
        p0, p1, p2, p3 = cur, cur[j1], nxt[j1], nxt
        tris.append(np.stack([np.stack([p0, p3, p2], axis=1), np.stack([p0, p2, p1], axis=1)], axis=1))
    return np.concatenate(tris).reshape(-1, 3, 3)


def sky_with_sun(width: int = 2048, height: int = 1024, sun_elevation_deg: float = 35.0,
                 sun_azimuth_deg: float = 60.0, sun_radius_deg: float = 0.5,
                 sun_radiance: float = 5.0e4) -> np.ndarray:
    """A linear f32 lat-long sky (row 0 = zenith, the EnvironmentLight layout of
    environment.rs:174-202): a smooth horizon-to-zenith gradient, a dim ground and a
    disc of the given angular radius and radiance around the sun direction."""
    theta = (np.arange(height) + 0.5) / height * math.pi
    phi = (np.arange(width) + 0.5) / width * 2.0 * math.pi
    T, Ph = np.meshgrid(theta, phi, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(Ph), np.cos(T), np.sin(T) * np.sin(Ph)], axis=-1)
    up = np.clip(d[..., 1], 0.0, 1.0)[..., None]
    horizon, zenith, ground = np.array([0.85, 0.9, 1.0]), np.array([0.25, 0.45, 0.95]), np.array([0.18, 0.16, 0.14])
    sky = horizon + (zenith - horizon) * np.sqrt(up)
    img = np.where(d[..., 1:2] >= 0.0, sky, ground)
    el, az = math.radians(sun_elevation_deg), math.radians(sun_azimuth_deg)
    sun = np.array([math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az)])
    in_disc = (d @ sun) >= math.cos(math.radians(sun_radius_deg))
    img[in_disc] = sun_radiance * np.array([1.0, 0.96, 0.9])
    return img.astype(np.float32)


def mesh_heavy_scene(size: int = 1024, tori: int = 64, rings: int = 32, tube: int = 64, seed: int = 1000,
                     env_width: int = 2048, env_height: int = 1024):
    """The mesh-heavy workload: a size x size Perlin fBm height field over a 100 x 100
    extent (2 (size-1)^2 triangles: 2,093,058 at 1024), `tori` tori of rings x tube x 2
    triangles at seeded positions, GGX microfacet materials (roughness U[0.05, 0.6],
    grey albedo U[0.2, 0.9]) and an HDR sky with a 0.5 degree, 5e4-radiance sun.
    Returns (scene, environment)."""
    rng = SampleRng(seed)
    extent = 100.0
    grad, perm = perlin_tables(seed)
    u = np.arange(size, dtype=np.float64) / float(size - 1) * 6.0
    U, V = np.meshgrid(u, u, indexing="xy")  # rows = z, columns = x
    base = np.stack([U.ravel(), np.full(U.size, 0.5), V.ravel()], axis=-1)
    h = np.zeros(U.size)
    for octave in range(4):  # fBm: sum_o 0.5^o noise(2^o p)
        h = h + 0.5 ** octave * perlin_noise(grad, perm, base * 2.0 ** octave)
    heights = h.reshape(size, size)

    def ggx() -> RayMaterial:
        a = rng.random_range(0.2, 0.9)
        r = rng.random_range(0.05, 0.6)
        return RayMaterial.ggx_microfacet((a, a, a), r)

    scene = RayScene()
    terrain = scene.add_material(ggx())
    scene.add_triangles_array(terrain, height_map_triangles(heights, extent, extent, 0.15 * extent))
    for _ in range(tori):
        c = (rng.random_range(-35.0, 35.0), rng.random_range(14.0, 24.0), rng.random_range(-35.0, 35.0))
        big = rng.random_range(1.5, 3.5)
        small = rng.random_range(0.3, 0.8)
        m = scene.add_material(ggx())
        scene.add_triangles_array(m, torus_triangles(c, small, big, rings, tube))
    scene.build_bvh()
    from .raytracing import EnvironmentLight
    return scene, EnvironmentLight(sky_with_sun(env_width, env_height))


def mesh_heavy_camera(width: int = 1920, height: int = 1080, grid: int = 8, max_depth: int = 8) -> RayCamera:
    """1920x1080, 8x8 stratified (64 spp), depth 8, looking over the height field at the tori."""
    return (RayCamera(width, width / height)
            .with_stratified_grid_width(grid)
            .with_max_depth(max_depth)
            .with_vertical_fov(40.0)
            .with_look_at((0.0, 38.0, 75.0), (0.0, 8.0, 0.0))
            .with_view_up((0.0, 1.0, 0.0)))


# ---------------------------------------------------- batched frames (cfg 3)
def batch_scene() -> tuple[RayScene, SamplingTargetList]:
    """The Cornell box with two MovingSpheres of radius 60 moving linearly over the
    shutter interval [0, 1)."""
    scene, lights = cornell_scene()
    orange = scene.add_material(RayMaterial.lambertian((0.8, 0.45, 0.1)))
    steel = scene.add_material(RayMaterial.metal((0.8, 0.85, 0.9), 0.05))
    scene.add_moving_sphere((400.0, 90.0, 160.0), (400.0, 170.0, 160.0), 60.0, orange)
    scene.add_moving_sphere((150.0, 330.0, 330.0), (230.0, 330.0, 300.0), 60.0, steel)
    scene.build_bvh()
    return scene, lights


def batch_cameras(frames: int = 64, width: int = 512, spp_cycle=(4, 8, 16, 32, 64), max_samples: int = 256,
                  threshold: float = 0.02, max_depth: int = 50) -> list:
    """`frames` square cameras orbiting the box centre (278, 278, 278) over -60..60 degrees,
    shutter [0, 1), adaptive random sampling whose minimum cycles through `spp_cycle` and
    whose cap is `max_samples`; each frame has its own RNG seed."""
    cams = []
    for i in range(frames):
        a = math.radians(-60.0 + 120.0 * i / max(frames - 1, 1))
        look_from = (278.0 + 1078.0 * math.sin(a), 278.0, 278.0 - 1078.0 * math.cos(a))
        spp = spp_cycle[i % len(spp_cycle)]
        cams.append(RayCamera(width, 1.0)
                    .with_adaptive_sampling(spp, max_samples, threshold)
                    .with_max_depth(max_depth)
                    .with_background((0.0, 0.0, 0.0))
                    .with_vertical_fov(40.0)
                    .with_look_at(look_from, (278.0, 278.0, 278.0))
                    .with_view_up((0.0, 1.0, 0.0))
                    .with_shutter_interval(0.0, 1.0)
                    .with_rng_seed(1 + i))
    return cams
