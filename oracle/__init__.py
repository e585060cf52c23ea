"""TEST INFRASTRUCTURE ONLY — ctypes access to the CPU oracle (gartus_oracle.hpp).

The oracle restates the reference's f64 renderer on the CPU.  Only tests/, the smoke
check in __graft_entry__ and bench.py's CPU-baseline leg may use it, and only as the
checker or the timed CPU baseline, never as the product path.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> Path:
    srcs = [HERE / "gartus_oracle.hpp", HERE / "oracle_capi.cpp", HERE.parent / "include" / "gartus_gpu.h"]
    if force or not LIB_PATH.exists() or any(s.stat().st_mtime > LIB_PATH.stat().st_mtime for s in srcs):
        subprocess.run(["make", "-C", str(HERE), "-B" if force else "all"], check=True, capture_output=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(str(LIB_PATH))
            vp, u32, i32, f64, u64 = C.c_void_p, C.c_uint32, C.c_int, C.c_double, C.c_uint64
            sig = {
                "orc_scene_create": (vp, [vp]),
                "orc_scene_destroy": (None, [vp]),
                "orc_scene_node_count": (u32, [vp]),
                "orc_scene_bvh": (None, [vp, vp, vp, vp]),
                "orc_trace_rays": (i32, [vp, vp, u32, f64, f64, i32, i32, vp, vp, vp, vp]),
                "orc_camera": (i32, [vp, vp, vp, vp, vp]),
                "orc_trace_primary": (i32, [vp, vp, u32, vp, vp, vp]),
                "orc_render": (i32, [vp, vp, u32, vp, vp, i32, u32, u32, u32, u32, u32, u32, i32, vp, vp, vp, vp]),
                "orc_pixel_seed": (u64, [u64, u32, u32]),
                "orc_slab": (i32, [vp, vp, f64, f64, vp]),
                "orc_pixel_trace": (C.c_int64, [vp, vp, u32, vp, vp, i32, u32, u32, u32, vp, vp, u64]),
                "orc_rng_u64": (None, [u64, u32, vp]),
                "orc_rng_double": (None, [u64, u32, vp]),
                "orc_perlin": (None, [u64, C.c_int, C.c_int, u32, vp, vp]),
                "orc_perlin_tables": (None, [u64, vp, vp]),
                "orc_intersect": (i32, [vp, vp, f64, f64, vp]),
                "orc_geometry_bounds": (None, [vp, vp]),
                "orc_geometry_pdf": (f64, [vp, vp, f64, vp]),
                "orc_lights_first_fraction": (f64, [vp, u32, vp, u64, u32]),
                "orc_env_pdf": (f64, [vp, vp]),
                "orc_ggx_d": (f64, [f64, f64]),
                "orc_ggx_g": (f64, [f64, f64, f64]),
                "orc_schlick": (f64, [f64, f64]),
                "orc_dielectric_reflectance": (f64, [f64, f64]),
                "orc_power_heuristic": (f64, [f64, f64]),
                "orc_adaptive_error": (f64, [vp, u32]),
                "orc_background": (None, [vp, vp, vp]),
                "orc_scatter": (i32, [vp, vp, vp, vp, i32, u64, vp, vp, vp]),
                "orc_scattering_pdf": (f64, [vp, vp, vp, vp, i32, vp]),
                "orc_cosine_pdf": (f64, [vp, vp]),
                "orc_image_sample": (None, [vp, f64, f64, vp]),
                "orc_medium_hit": (i32, [vp, vp, f64, f64, u64, vp, vp]),
                "orc_world_hit": (i32, [vp, vp, f64, f64, u64, vp]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
        return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


# Per-sample random streams of a render: the reference's (one per pixel) or the GPU
# throughput mode's (one per pixel and sample).
RNG_MODES = {"pixel": 0, "substreams": 1}


class OracleScene:
    """A RayScene loaded into the oracle (f64 and f32 copies, reference BVH built)."""

    def __init__(self, prims: np.ndarray, mats: np.ndarray, leaf_size: int = 4, images=(), media=(), meshes=(),
                 objects=()):
        from gartus_gb300 import abi
        from gartus_gb300.raytracing import _image_table, _media_table, _mesh_tables
        self._prims = np.ascontiguousarray(prims)
        self._mats = np.ascontiguousarray(mats)
        self._images = list(images)
        self._table = _image_table(self._images)
        self._media = list(media)
        self._mtable = _media_table(self._media)
        self._meshes, self._objects = list(meshes), list(objects)
        self._mesh_keep = _mesh_tables(self._meshes, self._objects)
        d = abi.gt_scene_desc()
        d.struct_size = C.sizeof(abi.gt_scene_desc)
        d.num_primitives = len(self._prims)
        d.primitives = self._prims.ctypes.data_as(C.POINTER(abi.gt_primitive))
        d.num_materials = len(self._mats)
        d.materials = self._mats.ctypes.data_as(C.POINTER(abi.gt_material))
        d.bvh_leaf_size = leaf_size
        d.num_images = len(self._images)
        d.images = self._table
        d.num_media = len(self._media)
        d.media = self._mtable
        d.num_meshes, d.meshes, d.num_objects, d.objects = self._mesh_keep[:4]
        self.h = lib().orc_scene_create(C.byref(d))
        if not self.h:
            raise ValueError("oracle rejected the scene")

    @classmethod
    def from_ray_scene(cls, scene) -> "OracleScene":
        return cls(scene.primitives_array(), scene.materials_array(), scene.leaf_size, scene.images(), scene.media(),
                   scene.mesh_list(), scene.object_list())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_scene_destroy(self.h)
            self.h = None

    def world_hit(self, ray, tmin: float = 0.001, tmax: float = float("inf"), seed: int = 0):
        """The world's closest hit (f64) of ray = (origin, direction[, time]), or None: a dict
        of t, point, normal, shading_normal, u, v, front_face, material."""
        r = np.zeros(7)
        r[:len(np.ravel(ray))] = np.ravel(ray)
        out = np.zeros(14)
        if not lib().orc_world_hit(self.h, _ptr(r), float(tmin), float(tmax), int(seed), _ptr(out)):
            return None
        return {"t": out[0], "point": out[1:4], "normal": out[4:7], "shading_normal": out[7:10],
                "u": out[10], "v": out[11], "front_face": bool(out[12]), "material": int(out[13])}

    def node_count(self) -> int:
        return lib().orc_scene_node_count(self.h)

    def bvh(self):
        n = self.node_count()
        bounds = np.zeros((n, 6))
        info = np.zeros((n, 3), dtype=np.uint32)
        idx = np.zeros(len(self._prims), dtype=np.uint32)
        lib().orc_scene_bvh(self.h, _ptr(bounds), _ptr(info), _ptr(idx))
        return bounds, info, idx

    def trace(self, rays: np.ndarray, t_min=0.001, t_max=np.inf, bruteforce=False, precision=1):
        from gartus_gb300 import abi
        rays = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 7)
        ids = np.empty(len(rays), dtype=np.int32)
        t = np.empty(len(rays))
        info = np.empty((len(rays), 8))
        st = abi.gt_bvh_stats()
        lib().orc_trace_rays(self.h, _ptr(rays), len(rays), t_min, t_max, int(bruteforce), precision, _ptr(ids),
                             _ptr(t), _ptr(info), C.byref(st))
        return ids, t, info, st.as_dict()

    def trace_primary(self, camera_desc, stride=1):
        from gartus_gb300 import abi
        w, h, spp = C.c_uint32(), C.c_uint32(), C.c_uint32()
        out = np.zeros(18)
        lib().orc_camera(C.byref(camera_desc), C.byref(w), C.byref(h), C.byref(spp), _ptr(out))
        n = ((w.value + stride - 1) // stride) * ((h.value + stride - 1) // stride)
        ids = np.empty(n, dtype=np.int32)
        t = np.empty(n)
        st = abi.gt_bvh_stats()
        lib().orc_trace_primary(self.h, C.byref(camera_desc), stride, _ptr(ids), _ptr(t), C.byref(st))
        return ids, t, st.as_dict()

    def pixel_trace(self, camera_desc, x: int, y: int, lights: np.ndarray | None = None, env=None,
                    precision: int = 1, rng: str = "pixel"):
        """The decision trace of pixel (x, y): (types, outcomes, values) of every discrete
        decision its samples take, in order (TraceEvent in gartus_oracle.hpp); rng as in
        render."""
        la = None if lights is None else np.ascontiguousarray(lights)
        envd = env.desc() if env is not None else None
        cap = 4096
        while True:
            kinds = np.zeros(2 * cap, dtype=np.int32)
            values = np.zeros(cap)
            n = lib().orc_pixel_trace(self.h, _ptr(la) if la is not None else None, len(la) if la is not None else 0,
                                      C.byref(envd) if envd is not None else None, C.byref(camera_desc), precision,
                                      RNG_MODES[rng], x, y, _ptr(kinds), _ptr(values), cap)
            if n < 0:
                raise ValueError("pixel outside the image")
            if n <= cap:
                return kinds[0:2 * n:2], kinds[1:2 * n:2], values[:n]
            cap = int(n)

    def render(self, camera_desc, lights: np.ndarray | None = None, env=None, precision: int = 1,
               threads: int = 1, window=(0, 0, 0, 0), aovs: bool = False, rng: str = "pixel"):
        """Renders (a window of) the image; returns (rgb, accepted[, albedo, normal]).  rng:
        "pixel" (each pixel's samples continue one stream, the reference) or "substreams"
        (sample s of pixel (x, y) draws from pixel_seed ^ sample_key(s))."""
        w, h, spp = camera_size(camera_desc)
        x0, y0, ww, hh = window
        ww = ww or w
        hh = hh or h
        rgb = np.zeros((hh, ww, 3))
        acc = np.zeros((hh, ww), dtype=np.uint32)
        alb = np.zeros((hh, ww, 3)) if aovs else None
        nrm = np.zeros((hh, ww, 3)) if aovs else None
        lp = None
        nl = 0
        if lights is not None:
            lights = np.ascontiguousarray(lights)
            lp = _ptr(lights)
            nl = len(lights)
        envd = C.byref(env.desc()) if env is not None else None
        rc = lib().orc_render(self.h, lp, nl, envd, C.byref(camera_desc), precision, RNG_MODES[rng], threads, x0,
                              y0, ww, hh, int(aovs), _ptr(rgb), _ptr(alb), _ptr(nrm), _ptr(acc))
        if rc != 0:
            raise RuntimeError(f"oracle render failed ({rc})")
        if aovs:
            return rgb, acc, alb, nrm
        return rgb, acc


def slab(ray, box, t_min: float, t_max: float):
    """RayTraversal::hit_bounds (bvh.rs:119-146): the entry distance of ray (origin,
    direction[, time]) into box (min xyz, max xyz), or None."""
    r = np.zeros(7)
    r[:len(np.ravel(ray))] = np.ravel(ray)
    b = np.ascontiguousarray(box, dtype=np.float64).reshape(6)
    e = C.c_double(0.0)
    return e.value if lib().orc_slab(_ptr(r), _ptr(b), float(t_min), float(t_max), C.byref(e)) else None


def camera_size(camera_desc):
    w, h, spp = C.c_uint32(), C.c_uint32(), C.c_uint32()
    out = np.zeros(18)
    lib().orc_camera(C.byref(camera_desc), C.byref(w), C.byref(h), C.byref(spp), _ptr(out))
    return w.value, h.value, spp.value


def camera_vectors(camera_desc) -> np.ndarray:
    w, h, spp = C.c_uint32(), C.c_uint32(), C.c_uint32()
    out = np.zeros(18)
    lib().orc_camera(C.byref(camera_desc), C.byref(w), C.byref(h), C.byref(spp), _ptr(out))
    return out.reshape(6, 3)


def image_sample(texture, u: float, v: float) -> np.ndarray:
    """ImageTexture::sample_linear (raytracing/texture.rs:148-155) of a
    gartus_gb300.raytracing.ImageTexture at (u, v): linear RGB, float64."""
    g = texture.to_struct()
    out = np.zeros(3)
    lib().orc_image_sample(C.byref(g), float(u), float(v), _ptr(out))
    return out


def medium_hit(boundary, density: float, ray, tmin: float, tmax: float, seed: int):
    """ConstantMedium::hit_with_rng of one medium (boundary a
    gartus_gb300.raytracing.MediumBoundary) on ray = (origin, direction[, time]) with a
    SampleRng seeded `seed`: (t or None, number of draws)."""
    m = boundary.to_struct(density, 0)
    r = np.zeros(7)
    r[:len(np.ravel(ray))] = np.ravel(ray)
    t = C.c_double()
    n = C.c_uint32()
    hit = lib().orc_medium_hit(C.byref(m), _ptr(r), float(tmin), float(tmax), int(seed), C.byref(t), C.byref(n))
    return (t.value if hit else None), n.value
