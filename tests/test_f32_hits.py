"""Check 1 on the f32 throughput walk that renders the image: primary-ray closest-hit
primitive ids through gt_trace_primary_f32 / gt_trace_rays_f32 (the eight-wide compressed
tree where the scene has one, f32 primitive tests) equal the f64 oracle's
(RayScene::hit, raytracing/scene.rs:1639-1657; traversal bvh.rs:306-399) on every ray.
Rays whose f32 decision may differ from f64 (a second candidate whose distance lies within
the two distances' estimated f32 errors of the closest, a hit point within f32 rounding of
an edge, a distance near t_min) are re-traced by the f64 walk; every other id is the f32
walk's own.  The counts of re-traced
rays are printed."""
import numpy as np
import pytest

import oracle
from gartus_gb300 import abi, scenes
from gartus_gb300.raytracing import PathTracer, RayMaterial, RayScene
from tests.test_gpu_parity import probe_rays

pytestmark = pytest.mark.gpu


def _check(ids, o_ids, refined, rep, name):
    print(f"{name}: {rep['rays']} rays, tree {'wide' if rep['tree'] == abi.GT_F32_TREE_WIDE else 'binary'} "
          f"({rep['wide_nodes']} nodes, depth {rep['wide_depth']}), re-traced in f64 {rep['refined']} "
          f"({rep['changed']} changed)")
    np.testing.assert_array_equal(ids, o_ids)
    assert rep["refined"] == int((refined > 0).sum())
    assert rep["changed"] == int((refined == 2).sum())


@pytest.mark.parametrize("name", ["final", "cornell", "bench"])
def test_f32_primary_ids_match_reference(gpu_context, name):
    if name == "final":
        scene, cam, stride = scenes.final_scene_ray_scene(), scenes.final_scene_camera(400, 1), 1
    elif name == "cornell":
        scene, cam, stride = scenes.cornell_scene()[0], scenes.cornell_camera(300, 1), 1
    else:  # the reference bench's probe set: every 4th pixel (benches/render_performance.rs:42-50)
        scene, cam, stride = scenes.render_performance_scene(), scenes.render_performance_camera(), 4
    pt = PathTracer(cam, context=gpu_context)
    ids, t, refined, rep = pt.trace_primary_f32(scene, stride)
    o_ids, o_t, _ = oracle.OracleScene.from_ray_scene(scene).trace_primary(cam.desc(), stride)
    _check(ids, o_ids, refined, rep, name)
    assert rep["tree"] == abi.GT_F32_TREE_WIDE
    # the f32 distances of rays kept in f32 agree with f64 to f32 rounding (the f32 ray is
    # the f64 ray rounded; at grazing angles on the r = 1000 ground that moves t by ~1e-4)
    keep = (refined == 0) & (ids >= 0)
    rel = np.abs(t[keep] - o_t[keep]) / np.abs(o_t[keep])
    print(f"{name}: relative t error of rays kept in f32: median {np.median(rel):.2e}, max {rel.max():.2e}")
    assert np.all(np.abs(t[keep] - o_t[keep]) <= 1e-3 * np.abs(o_t[keep]) + 1e-5)
    # near-edge and near-tie rays: observed 3.0% (final), 0.15% (Cornell), 1.5% (bench)
    assert rep["refined"] <= 0.05 * rep["rays"]


def test_f32_primary_ids_mesh_heavy(gpu_context):
    # The full 2,355,202-triangle mesh scene, every 16th pixel of the 1920x1080 frame.
    scene, _ = scenes.mesh_heavy_scene(env_width=8, env_height=4)
    cam = scenes.mesh_heavy_camera(1920, 1080, 1, 8)
    ids, t, refined, rep = PathTracer(cam, context=gpu_context).trace_primary_f32(scene, 16)
    o_ids, o_t, _ = oracle.OracleScene.from_ray_scene(scene).trace_primary(cam.desc(), 16)
    _check(ids, o_ids, refined, rep, "mesh_heavy")
    assert rep["tree"] == abi.GT_F32_TREE_WIDE and rep["wide_depth"] <= 32
    assert (ids >= 0).mean() > 0.5
    # 0.1-unit triangles seen from ~100 units: observed 8.8% within f32 reach of an edge
    assert rep["refined"] <= 0.12 * rep["rays"]


def test_f32_ids_randomized_scenes_and_binary_walk(gpu_context):
    # graphics/raytracing.rs:1340-1370's randomized scenes and probe rays, through the
    # wide walk and through the binary walk (GT_F32_TREE_BINARY).
    for seed in range(1, 17):
        scene = scenes.randomized_ray_scene(seed)
        rays = probe_rays(seed)
        o_ids, _, _, _ = oracle.OracleScene.from_ray_scene(scene).trace(rays)
        ids, _, refined, rep = scene.hit_rays_f32(rays, ctx=gpu_context)
        _check(ids, o_ids, refined, rep, f"randomized {seed} (wide)")
        scene.use_binary_f32_tree()
        ids_b, _, refined_b, rep_b = scene.hit_rays_f32(rays, ctx=gpu_context)
        assert rep_b["tree"] == abi.GT_F32_TREE_BINARY
        _check(ids_b, o_ids, refined_b, rep_b, f"randomized {seed} (binary)")


def test_f32_ids_edges_and_ties(gpu_context):
    # Rays aimed at the shared edges and vertices of a triangle fan and at the seam of two
    # coplanar quads: the f32 walk flags them and the f64 re-trace gives the reference's id.
    scene = RayScene()
    m = scene.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    c = np.array([0.0, 0.0, -5.0])
    for k in range(6):
        a0, a1 = 2 * np.pi * k / 6, 2 * np.pi * (k + 1) / 6
        scene.add_triangle(tuple(c), tuple(c + [np.cos(a0), np.sin(a0), 0]), tuple(c + [np.cos(a1), np.sin(a1), 0]), m)
    scene.add_quad((2.0, -1.0, -5.0), (1.0, 0.0, 0.0), (0.0, 2.0, 0.0), m)
    scene.add_quad((3.0, -1.0, -5.0), (1.0, 0.0, 0.0), (0.0, 2.0, 0.0), m)
    rays = []
    for k in range(6):  # spokes of the fan, and points just inside / outside them
        a = 2 * np.pi * k / 6
        for r in (0.0, 0.25, 0.5, 0.999999):
            for da in (0.0, 1e-9, -1e-9):
                p = c + r * np.array([np.cos(a + da), np.sin(a + da), 0.0])
                rays.append([0.1, 0.2, 0.0, p[0] - 0.1, p[1] - 0.2, p[2], 0.0])
    for y in np.linspace(-0.9, 0.9, 7):  # the quads' shared seam at x = 3
        for dx in (0.0, 1e-12, -1e-12):
            rays.append([0.0, 0.0, 0.0, 3.0 + dx, y, -5.0, 0.0])
    rays = np.array(rays)
    o_ids, _, _, _ = oracle.OracleScene.from_ray_scene(scene).trace(rays)
    ids, _, refined, rep = scene.hit_rays_f32(rays, ctx=gpu_context)
    _check(ids, o_ids, refined, rep, "edges")
    assert rep["refined"] > 0


def test_wide_and_binary_f32_images_agree(gpu_context):
    # The two f32 walks find the same closest hits, so the images agree to the last bit
    # except where two primitives are hit at exactly the same distance.
    scene = scenes.final_scene_ray_scene()
    cam = scenes.final_scene_camera(96, 4)
    wide = PathTracer(cam, context=gpu_context).render_hdr_image(scene)
    scene.use_binary_f32_tree()
    binary = PathTracer(cam, context=gpu_context).render_hdr_image(scene)
    same = (wide.pixels == binary.pixels).all(axis=2)
    assert same.mean() >= 0.995, same.mean()
    assert (wide.accepted == binary.accepted).all()
