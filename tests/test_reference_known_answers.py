"""More of the reference's own known-answer tests, restated: the slab test's edge cases
(raytracing/bvh.rs:712-770) on the oracle, the traversal statistics of a two-leaf tree
(bvh.rs:666-709), the gamma-2 and Reinhard display conversions (graphics/raytracing.rs:
553-557, 1504-1523), and the SurfaceScene to RayScene material policies (raytracing/scene.rs:
30-72, 1517-1547; raytracing/material.rs:2238-2262).  No GPU needed."""
import numpy as np
import pytest

import oracle
from gartus_gb300 import abi
from gartus_gb300.raytracing import (TONE_MAP_REINHARD, HdrImage, RayMaterial, RayScene, SurfaceMaterial,
                                     SurfaceRayMaterialMode, SurfaceScene, ToneMap, linear_color_to_rgb)

UNIT = (-1.0, -1.0, -1.0, 1.0, 1.0, 1.0)


def entry(origin, direction, box=UNIT, t_min=0.0, t_max=10.0):
    return oracle.slab(tuple(origin) + tuple(direction), box, t_min, t_max)


@pytest.mark.parametrize("d", [(1, 0, 0), (0, 1, 0), (0, 0, 1), (-1, 0, 0), (0, -1, 0), (0, 0, -1)])
def test_axis_parallel_rays_inside_bounds(d):  # bvh.rs:712-726
    assert entry((0, 0, 0), d) == 0.0


def test_parallel_rays_outside_slab_are_rejected():  # bvh.rs:728-742
    for o, d in [((0, 2, 0), (1, 0, 0)), ((0, 0, 2), (0, 1, 0)), ((2, 0, 0), (0, 0, 1))]:
        assert entry(o, d) is None


def test_slab_edge_cases():
    assert entry((0.25, -0.25, 0.5), (0, 0, 1)) == 0.0  # starting inside, bvh.rs:744-749
    assert entry((1.0, -2.0, 0.0), (0, 1, 0)) == 1.0  # on the boundary plane, bvh.rs:751-756
    assert entry((2.0, 2.0, 0.0), (-1, -1, 1)) is None  # one-point touch, bvh.rs:758-763
    assert entry((0.0, 0.0, -2.0), (0, 0, 1)) == 1.0  # zero direction components, bvh.rs:765-770
    assert entry((2.0, 0.0, -2.0), (0, 0, 1)) is None


def two_leaf_scene():
    # bvh.rs:666-709 builds leaves z in [1, 2] and [10, 11]; two spheres of radius 0.5
    # centred on the z axis have exactly those z extents and lie in one-per-leaf leaves.
    scene = RayScene()
    m = scene.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    scene.add_sphere((0.0, 0.0, 1.5), 0.5, m)
    scene.add_sphere((0.0, 0.0, 10.5), 0.5, m)
    scene.build_bvh_with_options(1)
    return scene


def test_two_leaf_traversal_stats():
    # A ray along +z meets the near leaf at t = 1; the far leaf's entry (10) is at or past
    # the closest hit, so it is skipped: tests 3, hits 3, leaf visits 1, candidates 1,
    # leaf hits 1 (bvh.rs:699-708).
    scene = two_leaf_scene()
    o = oracle.OracleScene.from_ray_scene(scene)
    ids, t, _, st = o.trace(np.array([[0, 0, 0, 0, 0, 1, 0.0]]), t_min=0.0, t_max=20.0)
    assert ids[0] == 0 and t[0] == 1.0
    assert (st["rays"], st["node_bounds_tests"], st["node_bounds_hits"], st["leaf_visits"],
            st["primitive_candidates"], st["leaf_hit_results"]) == (1, 3, 3, 1, 1, 1)
    assert st["max_stack_depth"] >= 1


def test_linear_color_to_rgb_applies_gamma_two():  # graphics/raytracing.rs:553-557
    assert linear_color_to_rgb((0.25, 0.0, 1.0)) == (128, 0, 255)


def test_reinhard_tone_mapping():  # graphics/raytracing.rs:1504-1523
    img = HdrImage(1, 1, np.array([[[4.0, 1.0, 0.25]]], dtype=np.float32))
    assert tuple(img.to_canvas()[0, 0]) == (255, 255, 128)
    tm = ToneMap().with_operator(TONE_MAP_REINHARD).with_gamma(1.0)
    assert tuple(img.to_canvas_tone_mapped(tm)[0, 0]) == (204, 128, 51)
    with pytest.raises(ValueError):
        ToneMap().with_gamma(0.0)


def _surface_scene():
    tri = np.array([[[-1, 0, -3], [1, 0, -3], [0, 1, -3]], [[-1, -1, -4], [1, -1, -4], [0, 0, -4]]], dtype=float)
    ss = SurfaceScene()
    ss.add_mesh(tri[:1], material=SurfaceMaterial(base_color=(0.8, 0.2, 0.1), specular_color=(0.6, 0.7, 0.8),
                                                  refractive_index=1.5))
    ss.add_mesh(tri[1:], material=SurfaceMaterial(base_color=(0.3, 0.4, 0.5), specular_color=(0.9, 0.9, 0.2)))
    return ss


def test_surface_material_modes():
    # SurfaceRayMaterialMode::convert (raytracing/scene.rs:56-67) with as_lambertian /
    # as_metal / as_dielectric (material.rs:2238-2262): one material per mesh, triangles
    # in mesh order.
    ss = _surface_scene()
    lam = ss.to_ray_scene().materials_array()
    assert list(lam["kind"]) == [abi.GT_MAT_LAMBERTIAN, abi.GT_MAT_LAMBERTIAN]
    np.testing.assert_array_equal(lam["color"], [[0.8, 0.2, 0.1], [0.3, 0.4, 0.5]])
    die = ss.to_ray_scene_with_material_mode(SurfaceRayMaterialMode.prefer_dielectric()).materials_array()
    assert list(die["kind"]) == [abi.GT_MAT_DIELECTRIC, abi.GT_MAT_LAMBERTIAN]
    assert die["param"][0] == 1.5
    met = ss.to_ray_scene_with_material_mode(SurfaceRayMaterialMode.prefer_metal(0.25)).materials_array()
    assert list(met["kind"]) == [abi.GT_MAT_METAL, abi.GT_MAT_METAL]
    np.testing.assert_array_equal(met["color"], [[0.6, 0.7, 0.8], [0.9, 0.9, 0.2]])
    assert list(met["param"]) == [0.25, 0.25]
    custom = SurfaceRayMaterialMode.custom(lambda m: RayMaterial.ggx_microfacet(m.base_color, 0.3))
    ggx = ss.to_ray_scene_with_material_mode(custom).materials_array()
    assert list(ggx["kind"]) == [abi.GT_MAT_GGX, abi.GT_MAT_GGX]
    np.testing.assert_array_equal(ggx["color"], [[0.8, 0.2, 0.1], [0.3, 0.4, 0.5]])
    prims = ss.to_ray_scene().primitives_array()
    assert list(prims["material"]) == [0, 1]
    np.testing.assert_array_equal(prims["geometry"]["p"][1], [-1, -1, -4, 1, -1, -4, 0, 0, -4])
    with pytest.raises(ValueError):
        SurfaceMaterial(refractive_index=0.0)
    with pytest.raises(TypeError):
        ss.to_ray_scene_with_material_mode(SurfaceRayMaterialMode.custom(lambda m: None))
