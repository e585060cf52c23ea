"""Seeded scene generators: the reference's own scenes and the synthetic workloads built
from them (raytracing/scenes.rs, benches/render_performance.rs, raytracing.rs tests).

Python floats are IEEE f64 without fused multiply-add, and math.sin/cos/sqrt call the C
library, so the geometry below is bit-identical to what the Rust generators produce.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from .raytracing import GLASS, RayCamera, RayMaterial, RayScene, SamplingTargetList

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
