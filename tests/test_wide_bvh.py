"""The eight-wide compressed tree of the f32 traversal (gartus_gb300/csrc/wide_bvh.cpp),
built on the CPU from the reference tree (raytracing/bvh.rs:233-288, 430-522) and checked
exactly: its leaf order is a permutation of the reference leaf order that keeps every
reference leaf's primitives together and in order, every slot's quantised planes bound
the f32 box of the reference node it stands for, and every reference node below the
root is one slot of one wide node.  The GPU tests check that the traversal over it finds
the reference's hits (tests/test_f32_hits.py)."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from gartus_gb300 import scenes
from gartus_gb300.raytracing import RayMaterial, RayScene
from tests.test_bvh_builder import grid_triangles

ROOT = Path(__file__).resolve().parents[1]
CODES = {1: "not built", 2: "leaf order is not a permutation", 3: "a plane does not bound its node",
         4: "a leaf slot's primitives differ from its reference leaf", 5: "internal children misnumbered",
         6: "an empty slot carries a child", 7: "a plane origin is not exact"}


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = tmp_path_factory.mktemp("wshim") / "libwideshim.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-I", str(ROOT / "include"), str(ROOT / "tests/shims/wide_shim.cpp"),
                    str(ROOT / "gartus_gb300/csrc/bvh_build.cpp"), str(ROOT / "gartus_gb300/csrc/wide_bvh.cpp"),
                    "-o", str(out)], check=True)
    lib = C.CDLL(str(out))
    lib.shim_wide.restype = C.c_int
    lib.shim_wide.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]
    return lib


def wide_check(shim, scene):
    prims = np.ascontiguousarray(scene.primitives_array())
    stats = np.zeros(5, dtype=np.uint32)
    code = shim.shim_wide(prims.ctypes.data_as(C.c_void_p), len(prims), scene.leaf_size,
                          stats.ctypes.data_as(C.c_void_p))
    return code, dict(zip(["nodes", "depth", "internal", "leaves", "empty"], map(int, stats)))


def cases():
    out = {"final_scene": scenes.final_scene_ray_scene(), "cornell": scenes.cornell_scene()[0],
           "bench": scenes.render_performance_scene(), "smoke": scenes.cornell_smoke_scene()[0]}
    for seed in (1, 5, 16):
        out[f"randomized_{seed}"] = scenes.randomized_ray_scene(seed)
    terrain = RayScene()
    m = terrain.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    terrain.add_triangles_array(m, grid_triangles(60, 4))
    out["terrain_7200"] = terrain
    far = RayScene()  # far from the origin: scales limited by f32's resolution there
    m = far.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    far.add_triangles_array(m, grid_triangles(12, 2) * 1e-3 + np.array([3.0e4, -2.0e4, 1.0e5]))
    out["far_small_triangles"] = far
    stack = RayScene()  # identical centroids
    m = stack.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    for i in range(37):
        stack.add_sphere((0.0, 0.0, 0.0), 1.0 + (i % 5) * 0.1, m)
    out["coincident_37"] = stack
    # a mesh's own tree (TriangleMesh, leaf size 4): the f32 wavefront walks object meshes
    # through the same wide form, their primitives in its leaf order
    torus = RayScene()
    m = torus.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    torus.add_triangles_array(m, scenes.torus_triangles((0.0, 0.0, 0.0), 0.35, 1.0, 32, 64))
    out["torus_mesh_4096"] = torus
    for leaf in (1, 2, 3):
        s = scenes.final_scene_ray_scene()
        s.build_bvh_with_options(leaf)
        out[f"final_leaf{leaf}"] = s
    return out


@pytest.mark.parametrize("name", list(cases().keys()))
def test_wide_tree_invariants(shim, name):
    code, st = wide_check(shim, cases()[name])
    assert code == 0, CODES.get(code, code)
    assert st["internal"] == st["nodes"] - 1  # every wide node but the root is one internal slot
    assert st["depth"] <= 32


def test_wide_tree_is_shallower_and_fuller(shim):
    scene = cases()["terrain_7200"]
    code, st = wide_check(shim, scene)
    assert code == 0
    # 7,200 triangles in leaves of <= 4: a binary tree of >= 1,800 leaves is >= 11 deep;
    # eight-wide nodes hold on average well over four children.
    assert st["depth"] <= 7
    assert (st["internal"] + st["leaves"]) / st["nodes"] > 6.0


def test_no_wide_form(shim):
    one = RayScene()
    m = one.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    one.add_sphere((0.0, 0.0, 0.0), 1.0, m)
    assert wide_check(shim, one)[0] == 1  # a leaf root keeps the binary walk
    big = scenes.final_scene_ray_scene()
    big.build_bvh_with_options(8)
    assert wide_check(shim, big)[0] == 1  # leaves of more than four primitives
