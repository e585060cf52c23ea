"""TriangleMesh and MatrixInstance in the oracle, pinned on the reference's tests
(graphics/raytracing.rs:1026-1047, 1929-2038) and on properties: the restated
Matrix::inverse against numpy, the mesh hit against a plain RayScene triangle, and an
instance against the same geometry placed by hand."""
import numpy as np
import pytest

import oracle
from gartus_gb300 import abi
from gartus_gb300.raytracing import (ImageTexture, MatrixInstance, NormalMap, RayGeometry, RayMaterial, RayScene,
                                     TriangleMesh, _lu_inverse)

TRI = [[0.0, 0.0, -1.0], [1.0, 0.0, -1.0], [0.0, 1.0, -1.0]]
DOWN = [0.25, 0.25, 0.0, 0.0, 0.0, -1.0]


def _world(*objects):
    scene = RayScene()
    for o in objects:
        scene.add_object(o)
    scene.build_bvh()
    return oracle.OracleScene.from_ray_scene(scene)


def _pixel_map(rgb):
    return NormalMap(ImageTexture(np.array(rgb, dtype=np.uint8).reshape(1, 1, 3)))


def test_mesh_texture_coordinates_and_shading_normals():  # graphics/raytracing.rs:1929-1958
    mesh = TriangleMesh([TRI], RayMaterial.lambertian((0.2, 0.2, 0.2)),
                        texcoords=[[(0.2, 0.4), (0.8, 0.4), (0.2, 0.9)]],
                        normals=[[(0.0, 1.0, 0.0)] * 3])
    h = _world(mesh).world_hit(DOWN, 0.0)
    assert h["t"] == pytest.approx(1.0) and h["u"] == pytest.approx(0.35) and h["v"] == pytest.approx(0.525)
    np.testing.assert_array_equal(h["normal"], [0.0, 0.0, 1.0])
    np.testing.assert_array_equal(h["shading_normal"], [0.0, 1.0, 0.0])


def test_mesh_applies_tangent_space_normal_map():  # graphics/raytracing.rs:1960-1988
    mat = RayMaterial.lambertian((0.2, 0.2, 0.2)).with_normal_map(_pixel_map((255, 128, 128)))
    mesh = TriangleMesh([TRI], mat, texcoords=[[(0.0, 0.0), (1.0, 0.0), (0.0, 1.0)]])
    assert _world(mesh).world_hit(DOWN, 0.0)["shading_normal"][0] > 0.7


def test_normal_map_green_channel_convention():  # graphics/raytracing.rs:1990-2006
    uv = [[(0.0, 0.0), (1.0, 0.0), (0.0, 1.0)]]
    up = TriangleMesh([TRI], RayMaterial.lambertian((0.2,) * 3).with_normal_map(_pixel_map((128, 255, 255))),
                      texcoords=uv)
    flipped_map = _pixel_map((128, 255, 255))
    flipped_map.flip_y = True
    down = TriangleMesh([TRI], RayMaterial.lambertian((0.2,) * 3).with_normal_map(flipped_map), texcoords=uv)
    assert _world(up).world_hit(DOWN, 0.0)["shading_normal"][1] > 0.7
    assert _world(down).world_hit(DOWN, 0.0)["shading_normal"][1] < -0.7


def test_mirrored_uv_handedness():  # graphics/raytracing.rs:2008-2038
    mat = RayMaterial.lambertian((0.2,) * 3).with_normal_map(_pixel_map((128, 255, 128)))
    mesh = TriangleMesh([TRI], mat, texcoords=[[(0.0, 0.0), (1.0, 0.0), (0.0, -1.0)]])
    assert _world(mesh).world_hit(DOWN, 0.0)["shading_normal"][1] < -0.7


def _translate(x, y, z):
    m = np.eye(4)
    m[:3, 3] = (x, y, z)
    return m


def test_matrix_instance_transforms_hits_and_normals():  # graphics/raytracing.rs:1026-1047
    sphere = TriangleMesh.from_geometry([RayGeometry.sphere((0.0, 0.0, -1.0), 0.5)], RayMaterial.lambertian((0.5,) * 3))
    inst = MatrixInstance(sphere, _translate(2.0, 0.0, 0.0) @ np.diag([2.0, 1.0, 1.0, 1.0]))
    h = _world(inst).world_hit([2.0, 0.0, 0.0, 0.0, 0.0, -1.0], 0.0)
    assert h["t"] == pytest.approx(0.5)
    assert h["point"][0] == pytest.approx(2.0) and h["point"][2] == pytest.approx(-0.5)
    assert h["normal"][2] == pytest.approx(1.0)
    np.testing.assert_array_equal(h["shading_normal"], h["normal"])


def test_instance_drops_vertex_normals_and_keeps_uv():
    # set_face_normal resets the shading normal (object.rs:455-467); (u, v) survive.
    mesh = TriangleMesh([TRI], RayMaterial.lambertian((0.2,) * 3), texcoords=[[(0.2, 0.4), (0.8, 0.4), (0.2, 0.9)]],
                        normals=[[(0.0, 1.0, 0.0)] * 3])
    h = _world(MatrixInstance(mesh, np.eye(4))).world_hit(DOWN, 0.0)
    assert h["u"] == pytest.approx(0.35) and h["v"] == pytest.approx(0.525)
    np.testing.assert_array_equal(h["shading_normal"], h["normal"])


def test_lu_inverse_matches_numpy_and_rejects_singular():
    rng = np.random.default_rng(3)
    for _ in range(50):
        m = rng.normal(size=(4, 4))
        np.testing.assert_allclose(np.array(_lu_inverse(m.tolist())), np.linalg.inv(m), rtol=1e-9, atol=1e-9)
    assert _lu_inverse(np.diag([1.0, 1.0, 0.0, 1.0]).tolist()) is None
    with pytest.raises(ValueError):
        MatrixInstance(TriangleMesh([TRI], RayMaterial.lambertian((0.5,) * 3)), np.zeros((4, 4)))


def test_mesh_matches_plain_triangles_and_placed_instance():
    # Without attributes a mesh hits exactly like the same triangles in the RayScene; a
    # translated instance like the mesh moved by hand.
    rng = np.random.default_rng(9)
    tris = rng.uniform(-1, 1, size=(40, 3, 3)) + np.array([0.0, 0.0, -4.0])
    mat = RayMaterial.lambertian((0.5, 0.5, 0.5))
    plain = RayScene()
    m = plain.add_material(mat)
    plain.add_triangles_array(m, tris)
    plain.build_bvh()
    o_plain = oracle.OracleScene.from_ray_scene(plain)
    o_mesh = _world(TriangleMesh(tris, mat))
    o_inst = _world(MatrixInstance(TriangleMesh(tris - np.array([0.5, -0.25, 1.0]), mat), _translate(0.5, -0.25, 1.0)))
    hits = 0
    for _ in range(300):
        ray = np.concatenate([rng.uniform(-0.5, 0.5, 3), rng.normal(size=3) * 0.3 + [0.0, 0.0, -1.0]])
        a, b, c = o_plain.world_hit(ray), o_mesh.world_hit(ray), o_inst.world_hit(ray)
        assert (a is None) == (b is None) == (c is None)
        if a is None:
            continue
        hits += 1
        assert a["t"] == b["t"] and np.array_equal(a["normal"], b["normal"])
        assert c["t"] == pytest.approx(a["t"], rel=1e-12)
        np.testing.assert_allclose(c["normal"], a["normal"], atol=1e-12)
    assert hits > 50


def test_scene_tables():
    img = ImageTexture(np.zeros((2, 2, 3), np.uint8))
    nm = NormalMap(img, strength=-3.0)
    assert nm.strength == 0.0  # with_strength clamps at 0
    mat = RayMaterial.ggx_microfacet((0.8, 0.8, 0.8), 0.3).with_normal_map(nm)
    mesh = TriangleMesh([TRI], mat)
    scene = RayScene()
    scene.add_object(mesh)
    scene.add_object(MatrixInstance(mesh, _translate(1, 2, 3)))
    assert len(scene.mesh_list()) == 1 and len(scene.object_list()) == 2
    mats = scene.materials_array()
    assert mats[0]["normal_map"] == 1 and scene.images() == [img]
    with pytest.raises(ValueError):
        RayMaterial.metal((0.5,) * 3, 0.1).with_normal_map(nm)
    with pytest.raises(TypeError):
        scene.add_object(RayGeometry.sphere((0, 0, 0), 1.0))
    assert abi.GT_NORMAL_MAP_NEGATIVE_Y == 1
