"""The product's host BVH builder (gartus_gb300/csrc/bvh_build.cpp) against the oracle's
restatement of FlatBvh::build (raytracing/bvh.rs:233-288, 430-522): the same nodes, in
the same pre-order, with the same bounds and the same primitive permutation."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from gartus_gb300 import abi, scenes
from gartus_gb300.raytracing import RayMaterial, RayScene

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = tmp_path_factory.mktemp("shim") / "libbvhshim.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-I", str(ROOT / "include"), str(ROOT / "tests/shims/bvh_shim.cpp"),
                    str(ROOT / "gartus_gb300/csrc/bvh_build.cpp"), "-o", str(out)], check=True)
    lib = C.CDLL(str(out))
    lib.shim_build.restype = C.c_int
    lib.shim_build.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32]
    return lib


def product_bvh(shim, scene, threads=0, cut=0):
    prims = np.ascontiguousarray(scene.primitives_array())
    cap = max(2 * len(prims), 1)
    n, depth = C.c_uint32(), C.c_uint32()
    bounds = np.zeros((cap, 6))
    info = np.zeros((cap, 3), dtype=np.uint32)
    order = np.zeros(len(prims), dtype=np.uint32)
    assert shim.shim_build(prims.ctypes.data_as(C.c_void_p), len(prims), scene.leaf_size, C.byref(n),
                           bounds.ctypes.data_as(C.c_void_p), info.ctypes.data_as(C.c_void_p),
                           order.ctypes.data_as(C.c_void_p), cap, C.byref(depth), threads, cut) == 0
    return bounds[: n.value], info[: n.value], order, depth.value


def grid_triangles(n, seed):
    """A jittered height-field of 2*n*n triangles (many equal centroids along rows)."""
    rng = np.random.default_rng(seed)
    h = rng.random((n + 1, n + 1)) * 0.3
    tris = []
    for z in range(n):
        for x in range(n):
            p00 = (x, h[z, x], z)
            p10 = (x + 1, h[z, x + 1], z)
            p01 = (x, h[z + 1, x], z + 1)
            p11 = (x + 1, h[z + 1, x + 1], z + 1)
            tris.append([p00, p01, p11])
            tris.append([p00, p11, p10])
    return np.array(tris, dtype=np.float64)


def cases():
    out = {"final_scene": scenes.final_scene_ray_scene(), "cornell": scenes.cornell_scene()[0],
           "bench": scenes.render_performance_scene()}
    for seed in (1, 7, 16):
        out[f"randomized_{seed}"] = scenes.randomized_ray_scene(seed)
    terrain = RayScene()
    m = terrain.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    terrain.add_triangles_array(m, grid_triangles(40, 3))
    out["terrain_3200"] = terrain
    # Identical centroids force the midpoint split (bvh.rs:442-444, 508-522).
    stack = RayScene()
    m = stack.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    for i in range(37):
        stack.add_sphere((0.0, 0.0, 0.0), 1.0 + (i % 5) * 0.1, m)
    out["coincident_37"] = stack
    for leaf in (1, 2, 8):
        s = scenes.final_scene_ray_scene()
        s.build_bvh_with_options(leaf)
        out[f"final_leaf{leaf}"] = s
    return out


# (threads, cut): the library's defaults (serial at these sizes), and the parallel build
# with subtrees of at most 16 primitives on four threads.
@pytest.mark.parametrize("threads,cut", [(0, 0), (4, 16)])
@pytest.mark.parametrize("name", list(cases().keys()))
def test_product_builder_matches_oracle(shim, name, threads, cut):
    scene = cases()[name]
    bounds, info, order, depth = product_bvh(shim, scene, threads, cut)
    o = oracle.OracleScene.from_ray_scene(scene)
    ob, oi, oo = o.bvh()
    assert len(bounds) == len(ob)
    np.testing.assert_array_equal(info, oi)
    np.testing.assert_array_equal(bounds, ob)
    np.testing.assert_array_equal(order, oo)
    assert 1 <= depth <= 61


def test_parallel_build_of_a_large_scene(shim):
    # 80,000 triangles: above the size where the library builds in parallel by default;
    # the parallel tree equals the oracle's and the serial build's node for node.
    scene = RayScene()
    m = scene.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    scene.add_triangles_array(m, grid_triangles(200, 11))
    par = product_bvh(shim, scene)
    ser = product_bvh(shim, scene, threads=1)
    for a, b in zip(par, ser):
        np.testing.assert_array_equal(a, b)
    ob, oi, oo = oracle.OracleScene.from_ray_scene(scene).bvh()
    np.testing.assert_array_equal(par[1], oi)
    np.testing.assert_array_equal(par[0], ob)
    np.testing.assert_array_equal(par[2], oo)


def test_empty_scene_has_no_nodes(shim):
    scene = RayScene()
    scene.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
    bounds, info, order, depth = product_bvh(shim, scene)
    assert len(bounds) == 0 and depth == 0
