"""Host-side mirror of gartus's path-tracing API over the C ABI (include/gartus_gpu.h).

The names, argument meanings and error behaviour follow the reference crate:
`RayMaterial` (raytracing/material.rs:2355-2508), `RayScene` (raytracing/scene.rs:1102-1696),
`SamplingTargetList` / `WeightedSamplingTargetList` (scene.rs:355-497),
`EnvironmentLight` (raytracing/environment.rs), `RayCamera` builder (graphics/camera.rs:
1034-1481), `PathTracer` (raytracing/renderer.rs:55-875) and `SurfaceScene::to_ray_scene`
(scene.rs:1517-1621).  Invalid input that makes the reference panic raises ValueError or a
GartusError carrying GT_ERR_INVALID_ARG.

Primitives are kept in a numpy structured array with gt_primitive's exact layout, so a
multi-million-triangle scene crosses the ABI without per-primitive Python objects.
"""
from __future__ import annotations

import copy
import ctypes as C
import math
import threading
import weakref
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import abi
from ._lib import GartusError, check, lib

GEOMETRY_DTYPE = np.dtype([("kind", "<u4"), ("reserved", "<u4"), ("p", "<f8", (9,))])
PRIMITIVE_DTYPE = np.dtype([("geometry", GEOMETRY_DTYPE), ("material", "<u4"), ("reserved", "<u4")])
MATERIAL_DTYPE = np.dtype([
    ("kind", "<u4"), ("texture_kind", "<u4"), ("color", "<f8", (3,)), ("param", "<f8"), ("tex", "<f8", (7,)),
    ("normal_map", "<u4"), ("normal_map_flags", "<u4"), ("normal_map_strength", "<f8"),
])
LIGHT_DTYPE = np.dtype([("geometry", GEOMETRY_DTYPE), ("weight", "<f8")])
assert PRIMITIVE_DTYPE.itemsize == C.sizeof(abi.gt_primitive)
assert MATERIAL_DTYPE.itemsize == C.sizeof(abi.gt_material)
assert LIGHT_DTYPE.itemsize == C.sizeof(abi.gt_light_target)

INFINITY = math.inf
SHADOW_ACNE_EPSILON = 0.001  # raytracing.rs:146
WIDESCREEN_ASPECT_RATIO = 16.0 / 9.0


def _vec(v, n=3) -> tuple:
    t = tuple(float(x) for x in v)
    if len(t) != n:
        raise ValueError(f"expected {n} components, got {len(t)}")
    return t


def _finite(*vals) -> bool:
    return all(math.isfinite(x) for v in vals for x in (v if isinstance(v, tuple) else (v,)))


# ------------------------------------------------------------------- geometry
@dataclass(frozen=True)
class RayGeometry:
    """RayGeometry (raytracing/object.rs:252-320)."""

    kind: int
    p: tuple

    @staticmethod
    def sphere(center, radius) -> "RayGeometry":
        return RayGeometry(abi.GT_GEOM_SPHERE, _vec(center) + (float(radius),) + (0.0,) * 5)

    @staticmethod
    def moving_sphere(center_start, center_end, radius) -> "RayGeometry":
        return RayGeometry(abi.GT_GEOM_MOVING_SPHERE, _vec(center_start) + _vec(center_end) + (float(radius), 0.0, 0.0))

    @staticmethod
    def triangle(p0, p1, p2) -> "RayGeometry":
        return RayGeometry(abi.GT_GEOM_TRIANGLE, _vec(p0) + _vec(p1) + _vec(p2))

    @staticmethod
    def quad(corner, u, v) -> "RayGeometry":
        return RayGeometry(abi.GT_GEOM_QUAD, _vec(corner) + _vec(u) + _vec(v))

    def to_abi(self) -> abi.gt_geometry:
        g = abi.gt_geometry()
        g.kind = self.kind
        for i, x in enumerate(self.p):
            g.p[i] = x
        return g


# ------------------------------------------------------------------- textures
class ImageTexture:
    """ImageTexture (raytracing/texture.rs:110-156) over the bitmap Texture of
    graphics/texture.rs: (H, W, 3) uint8 sRGB texels, row 0 at the top (t = 1), decoded to
    linear light as (c / 255)^2.  Texture::new defaults to nearest filtering and clamped
    coordinates (texture.rs:118-126); an empty image samples as cyan (texture.rs:150-152).
    The texels are copied into the scene when a material using the texture is compiled."""

    _FILTERS = {"nearest": abi.GT_FILTER_NEAREST, "linear": abi.GT_FILTER_LINEAR}
    _WRAPS = {"clamp": abi.GT_WRAP_CLAMP, "repeat": abi.GT_WRAP_REPEAT}

    def __init__(self, texels, filter: str = "nearest", wrap_s: str = "clamp", wrap_t: str = "clamp"):
        texels = np.asarray(texels)
        if texels.size == 0:
            texels = np.zeros((0, 0, 3), dtype=np.uint8)
        if texels.ndim != 3 or texels.shape[2] != 3 or texels.dtype != np.uint8:
            raise ValueError("image texels must be a (H, W, 3) uint8 array")
        if texels.shape[0] * texels.shape[1] > (1 << 28):
            raise ValueError("image texture has more than 2^28 texels")
        if filter not in self._FILTERS or wrap_s not in self._WRAPS or wrap_t not in self._WRAPS:
            raise ValueError("image filter must be nearest|linear and wraps clamp|repeat")
        self.texels = np.ascontiguousarray(texels)
        self.filter, self.wrap_s, self.wrap_t = filter, wrap_s, wrap_t

    def to_struct(self) -> abi.gt_image:
        g = abi.gt_image()
        g.height, g.width = self.texels.shape[0], self.texels.shape[1]
        g.rgb = self.texels.ctypes.data if self.texels.size else None
        g.filter = self._FILTERS[self.filter]
        g.wrap_s = self._WRAPS[self.wrap_s]
        g.wrap_t = self._WRAPS[self.wrap_t]
        return g


def _media_table(media: Sequence) -> "C.Array":
    """A gt_medium array for gt_scene_desc from (boundary, density, material id) entries."""
    arr = (abi.gt_medium * max(len(media), 1))()
    for i, (boundary, density, mat) in enumerate(media):
        arr[i] = boundary.to_struct(density, mat)
    return arr


class NormalMap:
    """NormalMap (raytracing/texture.rs:160-276): a tangent-space normal map over a bitmap
    (sampled with its filter and wraps, channels decoded as 2 c / 255 - 1), strength 1 and
    an OpenGL-style +Y green channel by default.  Attach with RayMaterial.with_normal_map."""

    def __init__(self, texture: ImageTexture, strength: float = 1.0, flip_y: bool = False):
        if not isinstance(texture, ImageTexture):
            raise TypeError("a normal map samples an ImageTexture")
        strength = float(strength)
        if not math.isfinite(strength):
            raise ValueError("normal-map strength must be finite")  # texture.rs:198-202
        self.texture = texture
        self.strength = max(strength, 0.0)
        self.flip_y = bool(flip_y)


def _lu_inverse(m) -> Optional[list]:
    """Matrix::inverse (gmath/matrix.rs:171-178): Doolittle LU with partial pivoting
    (lu_decomp, 285-338; a pivot below 1e-10 means singular) and forward / back substitution
    of the identity's columns (solve_with_lu, 351-400).  Row-major 4x4 lists of floats."""
    n = 4
    L = [[1.0 if i == j else 0.0 for j in range(n)] for i in range(n)]
    U = [list(map(float, row)) for row in m]
    P = list(range(n))
    for i in range(n):
        max_row, max_val = i, abs(U[i][i])
        for k in range(i + 1, n):
            if abs(U[k][i]) > max_val:
                max_val, max_row = abs(U[k][i]), k
        if max_val < 1e-10:
            return None
        if max_row != i:
            U[i], U[max_row] = U[max_row], U[i]
            P[i], P[max_row] = P[max_row], P[i]
            for k in range(i):
                L[i][k], L[max_row][k] = L[max_row][k], L[i][k]
        pivot = U[i][i]
        for j in range(i + 1, n):
            factor = U[j][i] / pivot
            L[j][i] = factor
            U[j][i] = 0.0
            for k in range(i + 1, n):
                U[j][k] = U[j][k] - factor * U[i][k]
    inv = [[0.0] * n for _ in range(n)]
    for col in range(n):
        y = [0.0] * n
        for i in range(n):
            acc = 0.0
            for j in range(i):
                acc += L[i][j] * y[j]
            y[i] = (1.0 if P[i] == col else 0.0) - acc
        x = [0.0] * n
        for i in reversed(range(n)):
            acc = 0.0
            for j in range(i + 1, n):
                acc += U[i][j] * x[j]
            x[i] = (y[i] - acc) / U[i][i]
        for i in range(n):
            inv[i][col] = x[i]
    return inv


class TriangleMesh:
    """TriangleMesh (raytracing/mesh.rs:149-360): triangles (N, 3, 3) in object space with
    one material, optional per-vertex texture coordinates (N, 3, 2) and vertex normals
    (N, 3, 3) (MeshTriangle::with_texcoords / with_vertex_normals, mesh.rs:44-54), and its
    own BVH (leaf size as BvhBuildOptions).  `present` (N,) optionally marks which triangles
    carry those attributes (bit 0 texture coordinates, bit 1 normals)."""

    def __init__(self, triangles, material: "RayMaterial", texcoords=None, normals=None, present=None,
                 leaf_size: int = 4):
        tri = np.asarray(triangles, dtype=np.float64)
        if tri.ndim != 3 or tri.shape[1:] != (3, 3):
            raise ValueError("triangles must be (N, 3, 3)")
        geoms = np.zeros(len(tri), dtype=GEOMETRY_DTYPE)
        geoms["kind"] = abi.GT_GEOM_TRIANGLE
        geoms["p"] = tri.reshape(-1, 9)
        self._init(geoms, material, texcoords, normals, present, leaf_size)

    @classmethod
    def from_geometry(cls, geometries: Sequence["RayGeometry"], material: "RayMaterial", leaf_size: int = 4):
        """Any RayGeometry list as one object (spheres and quads too), for instancing."""
        self = cls.__new__(cls)
        geoms = np.zeros(len(geometries), dtype=GEOMETRY_DTYPE)
        for i, g in enumerate(geometries):
            geoms[i]["kind"] = g.kind
            geoms[i]["p"] = g.p
        self._init(geoms, material, None, None, None, leaf_size)
        return self

    def _init(self, geoms, material, texcoords, normals, present, leaf_size):
        n = len(geoms)
        self.geometry = geoms
        self.material = material
        self.texcoords = None if texcoords is None else np.ascontiguousarray(texcoords, dtype=np.float64).reshape(n, 6)
        self.normals = None if normals is None else np.ascontiguousarray(normals, dtype=np.float64).reshape(n, 9)
        self.present = None if present is None else np.ascontiguousarray(present, dtype=np.uint8).reshape(n)
        for a in (self.texcoords, self.normals):
            if a is not None and not np.isfinite(a).all():
                raise ValueError("mesh attributes must be finite")
        self.leaf_size = max(int(leaf_size), 1)

    def __len__(self):
        return len(self.geometry)


class MatrixInstance:
    """MatrixInstance::new(object, transform) (raytracing/instance.rs:225-254): a mesh placed
    by a row-major 4x4 object-to-world matrix; its inverse is computed as Matrix::inverse
    does.  Raises ValueError where the reference returns None (no 4x4 inverse)."""

    def __init__(self, mesh: TriangleMesh, transform):
        m = np.asarray(transform, dtype=np.float64)
        if m.shape != (4, 4):
            raise ValueError("an instance transform is a 4x4 matrix")
        inv = _lu_inverse(m.tolist())
        if inv is None:
            raise ValueError("instance transform is not invertible")
        self.mesh = mesh
        self.transform = m.copy()
        self.inverse = np.array(inv)


def _mesh_tables(meshes: Sequence, objects: Sequence):
    """gt_mesh / gt_object arrays from (primitives, texcoords, normals, present, leaf) entries
    and (mesh index, transform or None, inverse) entries; the tuple ends with what must
    stay alive while the description is used."""
    marr = (abi.gt_mesh * max(len(meshes), 1))()
    keep = []
    for i, (prims, uv, vn, present, leaf) in enumerate(meshes):
        prims = np.ascontiguousarray(prims)
        keep += [prims, uv, vn, present]
        marr[i].num_primitives = len(prims)
        marr[i].bvh_leaf_size = leaf
        marr[i].primitives = prims.ctypes.data if len(prims) else None
        marr[i].texcoords = uv.ctypes.data if uv is not None else None
        marr[i].normals = vn.ctypes.data if vn is not None else None
        marr[i].attribute_flags = present.ctypes.data if present is not None else None
    oarr = (abi.gt_object * max(len(objects), 1))()
    for i, (mesh, xf, inv) in enumerate(objects):
        oarr[i].mesh = mesh
        oarr[i].transformed = 0 if xf is None else 1
        if xf is not None:
            for a, x in enumerate(np.ravel(xf)):
                oarr[i].transform[a] = float(x)
            for a, x in enumerate(np.ravel(inv)):
                oarr[i].inverse[a] = float(x)
    return len(meshes), marr, len(objects), oarr, keep


def _image_table(images: Sequence[ImageTexture]):
    """A gt_image array for gt_scene_desc (it points into the textures' own texels)."""
    arr = (abi.gt_image * max(len(images), 1))()
    for i, im in enumerate(images):
        arr[i] = im.to_struct()
    return arr


# ---------------------------------------------------------------------- media
class MediumBoundary:
    """The boundary of a ConstantMedium: a Sphere or a box_object (object.rs:930-976),
    optionally wrapped as Translate::new(RotateY::new(shape, degrees), offset)
    (instance.rs), the composition the reference's smoke scenes use."""

    def __init__(self, shape: int, p):
        self.shape = shape
        self.p = tuple(float(x) for x in p) + (0.0,) * (6 - len(p))
        self.degrees: Optional[float] = None
        self.offset: Optional[tuple] = None

    @staticmethod
    def sphere(center, radius) -> "MediumBoundary":
        return MediumBoundary(abi.GT_MEDIUM_SPHERE, _vec(center) + (float(radius),))

    @staticmethod
    def box(a, b) -> "MediumBoundary":
        return MediumBoundary(abi.GT_MEDIUM_BOX, _vec(a) + _vec(b))

    def rotate_y(self, degrees) -> "MediumBoundary":
        if self.degrees is not None or self.offset is not None:
            raise ValueError("a medium boundary takes one RotateY, inside its Translate")
        out = copy.copy(self)
        out.degrees = float(degrees)
        return out

    def translate(self, offset) -> "MediumBoundary":
        if self.offset is not None:
            raise ValueError("a medium boundary takes one Translate")
        out = copy.copy(self)
        out.offset = _vec(offset)
        return out

    def to_struct(self, density: float, material: int) -> abi.gt_medium:
        m = abi.gt_medium()
        m.shape = self.shape
        m.material = int(material)
        for i, x in enumerate(self.p):
            m.p[i] = x
        m.transform = 0
        if self.degrees is not None:
            m.rotate_y = self.degrees
            m.transform |= abi.GT_MEDIUM_ROTATE_Y
        if self.offset is not None:
            for i, x in enumerate(self.offset):
                m.translate[i] = x
            m.transform |= abi.GT_MEDIUM_TRANSLATE
        m.density = float(density)
        return m


# ------------------------------------------------------------------ materials
@dataclass(frozen=True)
class RayMaterial:
    """RayMaterial variants on the GPU path (raytracing/material.rs:2355-2363)."""

    kind: int
    color: tuple = (0.0, 0.0, 0.0)
    param: float = 0.0
    texture_kind: int = abi.GT_TEX_SOLID
    tex: tuple = (0.0,) * 7
    image: Optional[ImageTexture] = field(default=None, compare=False)
    normal_map: Optional[NormalMap] = field(default=None, compare=False)

    def with_normal_map(self, normal_map: NormalMap) -> "RayMaterial":
        """Lambertian / GgxMicrofacet::with_shared_normal_map (material.rs:456-460, 1505-1520):
        bends the shading normal at mesh triangles with texture coordinates."""
        if self.kind not in (abi.GT_MAT_LAMBERTIAN, abi.GT_MAT_GGX):
            raise ValueError("only Lambertian and GGX microfacet materials take a normal map")
        if not isinstance(normal_map, NormalMap):
            raise TypeError("with_normal_map takes a NormalMap")
        return RayMaterial(self.kind, self.color, self.param, self.texture_kind, self.tex, self.image, normal_map)

    @staticmethod
    def lambertian(albedo) -> "RayMaterial":
        albedo = _vec(albedo)
        if not _finite(albedo):
            raise ValueError("Lambertian albedo must be finite")
        return RayMaterial(abi.GT_MAT_LAMBERTIAN, albedo)

    @staticmethod
    def checker_lambertian(scale, even, odd) -> "RayMaterial":
        """Lambertian::checker (material.rs:443-446)."""
        return RayMaterial(abi.GT_MAT_LAMBERTIAN, (0.5, 0.5, 0.5), 0.0, abi.GT_TEX_CHECKER,
                           (float(scale),) + _vec(even) + _vec(odd))

    @staticmethod
    def _noise_tex(scale, variant: int, depth: int, seed: int) -> tuple:
        seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        depth = int(depth)
        if not math.isfinite(float(scale)) or not 0 <= depth <= 64:
            raise ValueError("noise texture needs a finite scale and a depth in 0..=64")
        return (float(scale), float(variant), float(depth), float(seed & 0xFFFFFFFF), float(seed >> 32), 0.0, 0.0)

    @staticmethod
    def noise_lambertian(scale, seed=1) -> "RayMaterial":
        """Lambertian::noise (material.rs:436-440): NoiseTexture::new(scale, seed)."""
        return RayMaterial(abi.GT_MAT_LAMBERTIAN, (0.5, 0.5, 0.5), 0.0, abi.GT_TEX_NOISE,
                           RayMaterial._noise_tex(scale, abi.GT_NOISE_PLAIN, 0, seed))

    @staticmethod
    def turbulence_lambertian(scale, depth=7, seed=1) -> "RayMaterial":
        """Lambertian::from_texture(NoiseTexture::turbulence(scale, depth, seed))."""
        return RayMaterial(abi.GT_MAT_LAMBERTIAN, (0.5, 0.5, 0.5), 0.0, abi.GT_TEX_NOISE,
                           RayMaterial._noise_tex(scale, abi.GT_NOISE_TURBULENCE, depth, seed))

    @staticmethod
    def marble_lambertian(scale, seed=1) -> "RayMaterial":
        """Lambertian::marble (material.rs:442-446): NoiseTexture::marble(scale, 7, seed)."""
        return RayMaterial(abi.GT_MAT_LAMBERTIAN, (0.5, 0.5, 0.5), 0.0, abi.GT_TEX_NOISE,
                           RayMaterial._noise_tex(scale, abi.GT_NOISE_MARBLE, 7, seed))

    @staticmethod
    def _textured(kind: int, texture: ImageTexture, param: float = 0.0) -> "RayMaterial":
        if not isinstance(texture, ImageTexture):
            raise TypeError("textured materials take an ImageTexture")
        return RayMaterial(kind, (0.0, 0.0, 0.0), param, abi.GT_TEX_IMAGE, (0.0,) * 7, texture)

    @staticmethod
    def textured_lambertian(texture: ImageTexture) -> "RayMaterial":
        """RayMaterial::textured_lambertian (material.rs:2393-2397)."""
        return RayMaterial._textured(abi.GT_MAT_LAMBERTIAN, texture)

    @staticmethod
    def textured_diffuse_light(texture: ImageTexture) -> "RayMaterial":
        """RayMaterial::textured_diffuse_light (material.rs:2419-2423)."""
        return RayMaterial._textured(abi.GT_MAT_DIFFUSE_LIGHT, texture)

    @staticmethod
    def textured_isotropic(texture: ImageTexture) -> "RayMaterial":
        """RayMaterial::textured_isotropic (material.rs:2445-2449)."""
        return RayMaterial._textured(abi.GT_MAT_ISOTROPIC, texture)

    @staticmethod
    def textured_henyey_greenstein(texture: ImageTexture, g) -> "RayMaterial":
        """HenyeyGreenstein::from_texture (material.rs:1264-1270)."""
        g = float(g)
        if not (math.isfinite(g) and abs(g) < 1.0):
            raise ValueError("Henyey-Greenstein anisotropy must be finite and in (-1, 1)")
        return RayMaterial._textured(abi.GT_MAT_HENYEY_GREENSTEIN, texture, g)

    @staticmethod
    def textured_ggx_microfacet(texture: ImageTexture, roughness) -> "RayMaterial":
        """GgxMicrofacet::from_texture (material.rs:1505-1511)."""
        if not math.isfinite(float(roughness)):
            raise ValueError("GGX microfacet material values must be finite")
        return RayMaterial._textured(abi.GT_MAT_GGX, texture, min(max(float(roughness), 0.0), 1.0))

    @staticmethod
    def diffuse_light(emit) -> "RayMaterial":
        emit = _vec(emit)
        if not _finite(emit):
            raise ValueError("diffuse light color must be finite")
        return RayMaterial(abi.GT_MAT_DIFFUSE_LIGHT, emit)

    @staticmethod
    def isotropic(albedo) -> "RayMaterial":
        albedo = _vec(albedo)
        if not _finite(albedo):
            raise ValueError("isotropic albedo must be finite")
        return RayMaterial(abi.GT_MAT_ISOTROPIC, albedo)

    @staticmethod
    def henyey_greenstein(albedo, g) -> "RayMaterial":
        """HenyeyGreenstein::new (material.rs:1175-1205): phase-function scattering around
        the incoming direction with anisotropy g in (-1, 1) (the reference panics outside)."""
        g = float(g)
        albedo = _vec(albedo)
        if not _finite(albedo):
            raise ValueError("Henyey-Greenstein albedo must be finite")
        if not (math.isfinite(g) and abs(g) < 1.0):
            raise ValueError("Henyey-Greenstein anisotropy must be finite and in (-1, 1)")
        return RayMaterial(abi.GT_MAT_HENYEY_GREENSTEIN, albedo, g)

    @staticmethod
    def ggx_microfacet(specular_color, roughness) -> "RayMaterial":
        c = _vec(specular_color)
        if not _finite(c, float(roughness)):
            raise ValueError("GGX microfacet material values must be finite")
        return RayMaterial(abi.GT_MAT_GGX, c, min(max(float(roughness), 0.0), 1.0))

    @staticmethod
    def metal(albedo, fuzz) -> "RayMaterial":
        c = _vec(albedo)
        if not _finite(c, float(fuzz)):
            raise ValueError("metal material values must be finite")
        return RayMaterial(abi.GT_MAT_METAL, c, min(max(float(fuzz), 0.0), 1.0))

    @staticmethod
    def dielectric(refraction_index) -> "RayMaterial":
        ri = float(refraction_index)
        if not (math.isfinite(ri) and ri > 0.0):
            raise ValueError("refractive index must be positive and finite")
        return RayMaterial(abi.GT_MAT_DIELECTRIC, (1.0, 1.0, 1.0), ri)

    def is_emissive(self) -> bool:  # material.rs:2555-2557
        return self.kind == abi.GT_MAT_DIFFUSE_LIGHT

    def to_record(self) -> tuple:
        nm = self.normal_map
        return (self.kind, self.texture_kind, self.color, self.param, self.tex, 0,
                int(nm.flip_y) * abi.GT_NORMAL_MAP_NEGATIVE_Y if nm else 0, nm.strength if nm else 0.0)


GLASS = 1.5  # RefractiveIndex::GLASS, graphics/lighting.rs:287


# -------------------------------------------------------------- sampling targets
class WeightedSamplingTargetList:
    """WeightedSamplingTargetList (raytracing/scene.rs:423-497)."""

    def __init__(self):
        self._targets: list[tuple[RayGeometry, float]] = []
        self._total = 0.0
        self._handles: dict = {}

    def add_target_weighted(self, geometry: RayGeometry, weight: float) -> None:
        weight = float(weight)
        if not (math.isfinite(weight) and weight > 0.0):
            raise ValueError("sampling target weight must be finite and positive")
        total = self._total + weight
        if not math.isfinite(total):
            raise ValueError("sampling target total weight must remain finite")
        self._total = total
        self._targets.append((geometry, weight))
        self._invalidate()

    def add_sphere_weighted(self, center, radius, weight):
        self.add_target_weighted(RayGeometry.sphere(center, radius), weight)

    def add_moving_sphere_weighted(self, c0, c1, radius, weight):
        self.add_target_weighted(RayGeometry.moving_sphere(c0, c1, radius), weight)

    def add_quad_weighted(self, corner, u, v, weight):
        self.add_target_weighted(RayGeometry.quad(corner, u, v), weight)

    def clear(self):
        self._targets.clear()
        self._total = 0.0
        self._invalidate()

    def __len__(self):
        return len(self._targets)

    def is_empty(self) -> bool:
        return not self._targets

    def total_weight(self) -> float:
        return self._total

    def to_array(self) -> np.ndarray:
        arr = np.zeros(len(self._targets), dtype=LIGHT_DTYPE)
        for i, (g, w) in enumerate(self._targets):
            arr[i]["geometry"]["kind"] = g.kind
            arr[i]["geometry"]["p"] = g.p
            arr[i]["weight"] = w
        return arr

    def _invalidate(self):
        for h in self._handles.values():
            h.close()
        self._handles = {}

    def _handle(self, ctx: "Context"):
        h = self._handles.get(id(ctx))
        if h is None or h.ctx is not ctx or not h.h:
            h = _LightsHandle(ctx, self.to_array())
            self._handles[id(ctx)] = h
        return h


class SamplingTargetList(WeightedSamplingTargetList):
    """SamplingTargetList (raytracing/scene.rs:355-421): every target has weight 1."""

    def add_sphere(self, center, radius):
        self.add_target_weighted(RayGeometry.sphere(center, radius), 1.0)

    def add_moving_sphere(self, c0, c1, radius):
        self.add_target_weighted(RayGeometry.moving_sphere(c0, c1, radius), 1.0)

    def add_quad(self, corner, u, v):
        self.add_target_weighted(RayGeometry.quad(corner, u, v), 1.0)

    def add_target(self, geometry: RayGeometry):
        self.add_target_weighted(geometry, 1.0)


# --------------------------------------------------------------------- context
class Context:
    """A CUDA device context with its own stream (gt_context)."""

    _default = None
    _default_lock = threading.Lock()

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().gt_context_create(int(device), C.byref(h)))
        self._h = h
        self.device = device
        self._dependents = weakref.WeakSet()  # scene / lights / environment handles, accumulators

    def _track(self, obj) -> None:
        self._dependents.add(obj)

    @classmethod
    def default(cls) -> "Context":
        with cls._default_lock:
            if cls._default is None:
                cls._default = Context(0)
            return cls._default

    @property
    def handle(self):
        return self._h

    def close(self):
        """Destroys the context after every handle made on it (their C objects must not
        outlive it)."""
        if self._h:
            for d in list(self._dependents):
                d.close()
            lib().gt_context_destroy(self._h)
            self._h = None


class _SceneHandle:
    def __init__(self, ctx: Context, prims: np.ndarray, mats: np.ndarray, leaf_size: int,
                 bvh_builder: int = abi.GT_BVH_REFERENCE_SAH, images: Sequence[ImageTexture] = (),
                 media: Sequence = (), meshes: Sequence = (), objects: Sequence = (),
                 f32_tree: int = abi.GT_F32_TREE_WIDE):
        self.ctx = ctx
        prims = np.ascontiguousarray(prims)
        mats = np.ascontiguousarray(mats)
        table = _image_table(images)
        mtable = _media_table(media)
        mesh_keep = _mesh_tables(meshes, objects)
        d = abi.gt_scene_desc()
        d.struct_size = C.sizeof(abi.gt_scene_desc)
        d.num_primitives = len(prims)
        d.primitives = prims.ctypes.data_as(C.POINTER(abi.gt_primitive))
        d.num_materials = len(mats)
        d.materials = mats.ctypes.data_as(C.POINTER(abi.gt_material))
        d.bvh_leaf_size = leaf_size
        d.bvh_builder = bvh_builder
        d.f32_tree = f32_tree
        d.num_images = len(images)
        d.images = table
        d.num_media = len(media)
        d.media = mtable
        d.num_meshes, d.meshes, d.num_objects, d.objects = mesh_keep[:4]
        h = C.c_void_p()
        check(lib().gt_scene_create(ctx.handle, C.byref(d), C.byref(h)))
        self.h = h
        ctx._track(self)

    def close(self):
        if self.h:
            lib().gt_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _LightsHandle:
    def __init__(self, ctx: Context, arr: np.ndarray):
        arr = np.ascontiguousarray(arr)
        h = C.c_void_p()
        check(lib().gt_lights_create(ctx.handle, arr.ctypes.data_as(C.c_void_p), len(arr), C.byref(h)))
        self.ctx = ctx
        self.h = h
        ctx._track(self)

    def close(self):
        if self.h:
            lib().gt_lights_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------------- scene
class RayScene:
    """RayScene (raytracing/scene.rs:1102-1696): material and primitive tables plus a
    lazily built BVH (the device copy is built on first use and reused)."""

    def __init__(self):
        self._materials: list[RayMaterial] = []
        self._chunks: list[np.ndarray] = []
        self._prims: Optional[np.ndarray] = np.zeros(0, dtype=PRIMITIVE_DTYPE)
        self._leaf_size = 4
        self._bvh_builder = abi.GT_BVH_REFERENCE_SAH
        self._f32_tree = abi.GT_F32_TREE_WIDE
        self._media: list = []
        self._meshes: list = []
        self._mesh_index: dict = {}
        self._objects: list = []
        self._handles: dict = {}

    # -- tables
    def add_material(self, material: RayMaterial) -> int:
        self._materials.append(material)
        self._invalidate()
        return len(self._materials) - 1

    def _check_material(self, material: int) -> None:
        if not (0 <= int(material) < len(self._materials)):
            raise ValueError("ray scene material id out of bounds")  # scene.rs:1158-1161

    def add_primitive(self, geometry: RayGeometry, material: int) -> None:
        self._check_material(material)
        rec = np.zeros(1, dtype=PRIMITIVE_DTYPE)
        rec["geometry"]["kind"] = geometry.kind
        rec["geometry"]["p"] = geometry.p
        rec["material"] = int(material)
        self._chunks.append(rec)
        self._invalidate()

    def add_primitives_array(self, prims: np.ndarray) -> None:
        """Bulk add_primitives (scene.rs:1174-1191) from a PRIMITIVE_DTYPE array."""
        prims = np.asarray(prims, dtype=PRIMITIVE_DTYPE)
        if len(prims) and (prims["material"].max() >= len(self._materials)):
            raise ValueError("ray scene material id out of bounds")
        self._chunks.append(prims.copy())
        self._invalidate()

    def add_triangles_array(self, material: int, vertices: np.ndarray) -> None:
        """add_triangles (scene.rs:1313-1324) from an (N, 3, 3) float64 array."""
        self._check_material(material)
        v = np.asarray(vertices, dtype=np.float64).reshape(-1, 9)
        rec = np.zeros(len(v), dtype=PRIMITIVE_DTYPE)
        rec["geometry"]["kind"] = abi.GT_GEOM_TRIANGLE
        rec["geometry"]["p"] = v
        rec["material"] = int(material)
        self._chunks.append(rec)
        self._invalidate()

    def add_sphere(self, center, radius, material):
        self.add_primitive(RayGeometry.sphere(center, radius), material)

    def add_moving_sphere(self, center_start, center_end, radius, material):
        self.add_primitive(RayGeometry.moving_sphere(center_start, center_end, radius), material)

    def add_quad(self, corner, u, v, material):
        self.add_primitive(RayGeometry.quad(corner, u, v), material)

    def add_triangle(self, p0, p1, p2, material):
        self.add_primitive(RayGeometry.triangle(p0, p1, p2), material)

    def add_sphere_with_material(self, center, radius, material: RayMaterial) -> int:
        mid = self.add_material(material)
        self.add_sphere(center, radius, mid)
        return mid

    def add_moving_sphere_with_material(self, c0, c1, radius, material: RayMaterial) -> int:
        mid = self.add_material(material)
        self.add_moving_sphere(c0, c1, radius, mid)
        return mid

    def add_quad_with_material(self, corner, u, v, material: RayMaterial) -> int:
        mid = self.add_material(material)
        self.add_quad(corner, u, v, mid)
        return mid

    # -- world objects
    def add_object(self, obj) -> int:
        """A TriangleMesh, or a MatrixInstance of one, after the RayScene's surfaces in the
        world's hit order (HittableList, scene.rs:177-197; the media come after them).  The
        mesh's material joins the material table.  Returns the object index."""
        mesh, xf, inv = (obj.mesh, obj.transform, obj.inverse) if isinstance(obj, MatrixInstance) else (obj, None, None)
        if not isinstance(mesh, TriangleMesh):
            raise TypeError("a world object is a TriangleMesh or a MatrixInstance of one")
        key = id(mesh)
        if key not in self._mesh_index:
            mid = self.add_material(mesh.material)
            self._mesh_index[key] = (len(self._meshes), mid)
            self._meshes.append(mesh)
        self._objects.append((self._mesh_index[key][0], xf, inv))
        self._invalidate()
        return len(self._objects) - 1

    def mesh_list(self) -> list:
        """(primitives, texcoords, normals, present, leaf size) per mesh, materials resolved."""
        out = []
        for mesh in self._meshes:
            prims = np.zeros(len(mesh), dtype=PRIMITIVE_DTYPE)
            prims["geometry"] = mesh.geometry
            prims["material"] = self._mesh_index[id(mesh)][1]
            out.append((prims, mesh.texcoords, mesh.normals, mesh.present, mesh.leaf_size))
        return out

    def object_list(self) -> list:
        return list(self._objects)

    # -- animation
    def update_primitives(self, first: int, primitives: np.ndarray) -> None:
        """Replaces primitives [first, first + len) in place, keeping the scene's device
        copies (gt_scene_update_primitives): the per-frame move of an animation's dynamic
        geometry, which the reference rebuilds as the dynamic layer of a HittableLayers
        split (scene.rs:227-351).  A scene using the GPU-built tree has it refitted on the
        device; the reference tree is rebuilt on the host."""
        arr = np.ascontiguousarray(primitives, dtype=PRIMITIVE_DTYPE)
        prims = self.primitives_array()
        first = int(first)
        if first < 0 or first + len(arr) > len(prims):
            raise ValueError("primitive range out of bounds")
        if len(arr) and int(arr["material"].max()) >= len(self._materials):
            raise ValueError("ray scene material id out of bounds")  # scene.rs:1158-1161
        for h in list(self._handles.values()):
            if h.h:
                check(lib().gt_scene_update_primitives(h.h, first, len(arr), arr.ctypes.data_as(C.c_void_p)))
        prims[first:first + len(arr)] = arr

    # -- participating media
    def add_constant_medium(self, boundary: MediumBoundary, density, albedo) -> int:
        """ConstantMedium::new(boundary, density, albedo) (volume/medium.rs:30-39): an
        Isotropic phase function.  Media follow the surfaces in the world's hit order, in
        the order they are added (HittableList, scene.rs:177-197).  Returns the medium index."""
        return self.add_medium_with_phase_function(boundary, density, RayMaterial.isotropic(albedo))

    def add_medium_with_phase_function(self, boundary: MediumBoundary, density, material: RayMaterial) -> int:
        """ConstantMedium::with_phase_function (volume/medium.rs:71-81)."""
        density = float(density)
        if not (math.isfinite(density) and density > 0.0):
            raise ValueError("medium density must be positive and finite")  # medium.rs:93-96
        if not isinstance(boundary, MediumBoundary):
            raise TypeError("a medium boundary is a MediumBoundary")
        if len(self._media) >= 64:
            raise ValueError("at most 64 media per scene")
        mid = self.add_material(material)
        self._media.append((boundary, density, mid))
        self._invalidate()
        return len(self._media) - 1

    def media(self) -> list:
        """(boundary, density, material id) per medium, in hit order."""
        return list(self._media)

    # -- BVH options
    def build_bvh(self) -> None:
        self.build_bvh_with_options(4)

    def use_gpu_bvh(self, enabled: bool = True) -> "RayScene":
        """The f32 path traverses a linear BVH built on the GPU at upload (gt_bvh_builder
        GT_BVH_GPU_LBVH) instead of the reference's SAH tree, which is then built on the
        host only for f64 rendering and traversal statistics.  For large scenes."""
        builder = abi.GT_BVH_GPU_LBVH if enabled else abi.GT_BVH_REFERENCE_SAH
        if builder != self._bvh_builder:
            self._bvh_builder = builder
            self._invalidate()
        return self

    def use_binary_f32_tree(self, enabled: bool = True) -> "RayScene":
        """The f32 path walks the reference's binary tree (gt_f32_tree GT_F32_TREE_BINARY)
        instead of the eight-wide compressed tree collapsed from it.  Same hits; for
        comparisons."""
        tree = abi.GT_F32_TREE_BINARY if enabled else abi.GT_F32_TREE_WIDE
        if tree != self._f32_tree:
            self._f32_tree = tree
            self._invalidate()
        return self

    def build_bvh_with_options(self, leaf_size: int = 4) -> None:
        """BvhBuildOptions::with_leaf_size clamps 0 to 1 (bvh.rs:73-77)."""
        self._leaf_size = max(int(leaf_size), 1)
        self._invalidate()

    def with_bvh(self) -> "RayScene":
        self.build_bvh()
        return self

    # -- views
    def materials(self) -> list[RayMaterial]:
        return list(self._materials)

    def primitives_array(self) -> np.ndarray:
        if self._chunks:
            parts = [self._prims] + self._chunks if len(self._prims) else self._chunks
            self._prims = np.concatenate(parts) if len(parts) > 1 else parts[0]
            self._chunks = []
        return self._prims

    def materials_array(self) -> np.ndarray:
        arr = np.zeros(len(self._materials), dtype=MATERIAL_DTYPE)
        index = {id(im): k for k, im in enumerate(self.images())}
        for i, m in enumerate(self._materials):
            arr[i] = m.to_record()
            if m.image is not None:
                arr[i]["tex"][0] = index[id(m.image)]
            if m.normal_map is not None:
                arr[i]["normal_map"] = 1 + index[id(m.normal_map.texture)]
        return arr

    def images(self) -> list:
        """The distinct ImageTextures of the materials, in first-use order (the scene's
        gt_image table; a GT_TEX_IMAGE material's tex[0] indexes it)."""
        out, seen = [], set()
        for m in self._materials:
            for im in (m.image, m.normal_map.texture if m.normal_map is not None else None):
                if im is not None and id(im) not in seen:
                    seen.add(id(im))
                    out.append(im)
        return out

    @property
    def leaf_size(self) -> int:
        return self._leaf_size

    def __len__(self) -> int:
        return len(self.primitives_array())

    def is_empty(self) -> bool:
        return len(self) == 0

    def material_count(self) -> int:
        return len(self._materials)

    def emissive_targets(self) -> SamplingTargetList:
        """RayScene::emissive_targets (scene.rs:1401-1423)."""
        targets = SamplingTargetList()
        prims = self.primitives_array()
        for rec in prims:
            if self._materials[int(rec["material"])].is_emissive():
                targets.add_target(RayGeometry(int(rec["geometry"]["kind"]), tuple(float(x) for x in rec["geometry"]["p"])))
        return targets

    # -- device handle
    def _invalidate(self):
        for h in self._handles.values():
            h.close()
        self._handles = {}

    def _handle(self, ctx: Context) -> _SceneHandle:
        h = self._handles.get(id(ctx))
        if h is None or h.ctx is not ctx or not h.h:
            h = _SceneHandle(ctx, self.primitives_array(), self.materials_array(), self._leaf_size,
                             self._bvh_builder, self.images(), self._media, self.mesh_list(), self._objects,
                             self._f32_tree)
            self._handles[id(ctx)] = h
        return h

    def bvh_node_count(self, ctx: Optional[Context] = None) -> int:
        n = C.c_uint32()
        check(lib().gt_scene_bvh_node_count(self._handle(ctx or Context.default()).h, C.byref(n)))
        return n.value

    def hit_rays(self, rays: np.ndarray, t_min: float = SHADOW_ACNE_EPSILON, t_max: float = INFINITY,
                 ctx: Optional[Context] = None):
        """Closest hits of (N, 7) rays {origin, direction, time} in f64 with the summed
        BvhTraversalStats (scene.rs:1474-1492).  Returns (prim_ids, t, stats)."""
        rays = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 7)
        ids = np.empty(len(rays), dtype=np.int32)
        t = np.empty(len(rays), dtype=np.float64)
        st = abi.gt_bvh_stats()
        check(lib().gt_trace_rays(self._handle(ctx or Context.default()).h, rays.ctypes.data_as(C.c_void_p),
                                  len(rays), float(t_min), float(t_max), ids.ctypes.data_as(C.c_void_p),
                                  t.ctypes.data_as(C.c_void_p), C.byref(st)))
        return ids, t, st.as_dict()

    def hit_rays_f32(self, rays: np.ndarray, t_min: float = SHADOW_ACNE_EPSILON, t_max: float = INFINITY,
                     ctx: Optional[Context] = None):
        """hit_rays through the renderer's f32 walk, with near-tie rays re-traced in f64
        (gt_trace_rays_f32).  Returns (prim_ids, t, refined, report): refined is 0 for an
        f32 result, 1 for an f64 re-trace that kept the primitive, 2 for one that changed it."""
        rays = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 7)
        ids = np.empty(len(rays), dtype=np.int32)
        t = np.empty(len(rays), dtype=np.float64)
        refined = np.empty(len(rays), dtype=np.uint8)
        rep = abi.gt_trace_report()
        rep.struct_size = C.sizeof(abi.gt_trace_report)
        check(lib().gt_trace_rays_f32(self._handle(ctx or Context.default()).h, rays.ctypes.data_as(C.c_void_p),
                                      len(rays), float(t_min), float(t_max), ids.ctypes.data_as(C.c_void_p),
                                      t.ctypes.data_as(C.c_void_p), refined.ctypes.data_as(C.c_void_p),
                                      C.byref(rep)))
        return ids, t, refined, rep.as_dict()

    def bvh_traversal_stats_for_rays(self, rays: np.ndarray, t_min: float = SHADOW_ACNE_EPSILON,
                                     t_max: float = INFINITY) -> dict:
        return self.hit_rays(rays, t_min, t_max)[2]


# ---------------------------------------------------------------- environment
class EnvironmentLight:
    """EnvironmentLight (raytracing/environment.rs:22-202).  `texels` is (H, W, 3): uint8
    for the reference's 8-bit gamma-2 canvas, float32 for the linear HDR extension.
    Row 0 is the zenith."""

    def __init__(self, texels: np.ndarray):
        texels = np.asarray(texels)
        if texels.ndim != 3 or texels.shape[2] != 3 or texels.shape[0] == 0 or texels.shape[1] == 0:
            raise ValueError("environment texels must be a non-empty (H, W, 3) array")
        if texels.dtype == np.uint8:
            self.format = abi.GT_ENV_SRGB8
        else:
            texels = texels.astype(np.float32)
            if not np.isfinite(texels).all():
                raise ValueError("environment texels must be finite")
            self.format = abi.GT_ENV_RGB32F
        self.texels = np.ascontiguousarray(texels)
        self._handles: dict = {}

    @property
    def width(self) -> int:
        return self.texels.shape[1]

    @property
    def height(self) -> int:
        return self.texels.shape[0]

    def desc(self) -> abi.gt_environment_desc:
        d = abi.gt_environment_desc()
        d.struct_size = C.sizeof(abi.gt_environment_desc)
        d.format = self.format
        d.width = self.width
        d.height = self.height
        d.texels = self.texels.ctypes.data_as(C.c_void_p)
        return d

    def _handle(self, ctx: Context):
        h = self._handles.get(id(ctx))
        if h is None or h.ctx is not ctx or not h.h:
            h = _EnvHandle(ctx, self)
            self._handles[id(ctx)] = h
        return h


class _EnvHandle:
    def __init__(self, ctx: Context, env: EnvironmentLight):
        d = env.desc()
        h = C.c_void_p()
        check(lib().gt_environment_create(ctx.handle, C.byref(d), C.byref(h)))
        self.ctx = ctx
        self.h = h
        ctx._track(self)

    def close(self):
        if self.h:
            lib().gt_environment_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------------- camera
PixelSampleMode = {"random": abi.GT_SAMPLE_RANDOM, "stratified": abi.GT_SAMPLE_STRATIFIED,
                   "grid": abi.GT_SAMPLE_STRATIFIED_GRID}


class RayCamera:
    """RayCamera builder (graphics/camera.rs:1034-1481).  Each with_* returns a new camera."""

    def __init__(self, image_width: int, aspect_ratio: float):
        """RayCamera::new (camera.rs:1034-1065): the reference's defaults, as gt_camera_default
        writes them (a host-side restatement, so that a camera can be described without the
        device library)."""
        if int(image_width) <= 0:
            raise GartusError(abi.GT_ERR_INVALID_ARG, "image width must be positive")
        if not (math.isfinite(aspect_ratio) and aspect_ratio > 0.0):
            raise GartusError(abi.GT_ERR_INVALID_ARG, "aspect ratio must be positive and finite")
        d = abi.gt_camera_desc()
        d.struct_size = C.sizeof(abi.gt_camera_desc)
        d.image_width, d.aspect_ratio = int(image_width), float(aspect_ratio)
        d.samples_per_pixel, d.pixel_sample_mode, d.grid_width = 1, abi.GT_SAMPLE_RANDOM, 1
        d.direct_lighting_mode, d.light_pdf_weight = abi.GT_DIRECT_CURRENT_PATH_CONTINUATION, 0.5
        d.max_depth, d.russian_roulette_min_depth, d.rng_seed = 10, 5, 1
        d.vertical_fov = 90.0
        d.lookat[2], d.view_up[1] = -1.0, 1.0
        d.focus_distance, d.shutter_end = 1.0, 1.0
        d.background_kind = abi.GT_BG_CONSTANT
        d.background[0], d.background[1], d.background[2] = 0.70, 0.80, 1.00
        self._d = d

    @classmethod
    def from_desc(cls, d: abi.gt_camera_desc) -> "RayCamera":
        cam = cls.__new__(cls)
        cam._d = copy.copy(d)
        return cam

    def desc(self) -> abi.gt_camera_desc:
        return self._d

    def _with(self, **kw) -> "RayCamera":
        d = abi.gt_camera_desc()
        C.pointer(d)[0] = self._d
        for k, v in kw.items():
            if isinstance(v, tuple):
                arr = getattr(d, k)
                for i, x in enumerate(v):
                    arr[i] = x
            else:
                setattr(d, k, v)
        return RayCamera.from_desc(d)

    def with_samples_per_pixel(self, spp: int):
        return self._with(samples_per_pixel=max(int(spp), 1))

    def with_pixel_sample_mode(self, mode: int):
        return self._with(pixel_sample_mode=int(mode))

    def with_stratified_sampling(self):
        return self._with(pixel_sample_mode=abi.GT_SAMPLE_STRATIFIED)

    def with_stratified_grid_width(self, grid_width: int):
        g = max(int(grid_width), 1)
        return self._with(samples_per_pixel=g * g, pixel_sample_mode=abi.GT_SAMPLE_STRATIFIED_GRID, grid_width=g)

    def with_adaptive_sampling(self, min_samples: int, max_samples: int, error_threshold: float):
        thr = float(error_threshold)
        if not (math.isfinite(thr) and thr > 0.0):
            raise ValueError("adaptive sampling error threshold must be positive and finite")
        mn = max(int(min_samples), 1)
        mx = max(int(max_samples), mn)
        return self._with(adaptive=1, adaptive_min_samples=mn, adaptive_max_samples=mx,
                          adaptive_error_threshold=thr, samples_per_pixel=mx)

    def without_adaptive_sampling(self):
        return self._with(adaptive=0)

    def with_direct_lighting_mode(self, mode: int):
        w = 0.5 if mode == abi.GT_DIRECT_CURRENT_PATH_CONTINUATION else 0.0
        return self._with(direct_lighting_mode=int(mode), light_pdf_weight=w)

    def with_light_pdf_weight(self, weight: float):
        weight = float(weight)
        if not math.isfinite(weight):
            raise ValueError("light PDF weight must be finite")
        return self._with(direct_lighting_mode=abi.GT_DIRECT_CURRENT_PATH_CONTINUATION,
                          light_pdf_weight=min(max(weight, 0.0), 1.0))

    def with_max_depth(self, depth: int):
        return self._with(max_depth=int(depth))

    def with_russian_roulette_min_depth(self, depth: int):
        return self._with(russian_roulette_min_depth=int(depth))

    def without_russian_roulette(self):
        return self._with(russian_roulette_min_depth=-1)

    def with_rng_seed(self, seed: int):
        return self._with(rng_seed=int(seed) & 0xFFFFFFFFFFFFFFFF)

    def with_vertical_fov(self, fov: float):
        return self._with(vertical_fov=float(fov))

    def with_look_at(self, lookfrom, lookat):
        return self._with(lookfrom=_vec(lookfrom), lookat=_vec(lookat))

    def with_view_up(self, vup):
        return self._with(view_up=_vec(vup))

    def with_defocus_angle(self, angle: float):
        return self._with(defocus_angle=float(angle))

    def with_focus_distance(self, dist: float):
        return self._with(focus_distance=float(dist))

    def with_shutter_interval(self, start: float, end: float):
        if not (math.isfinite(start) and math.isfinite(end) and start <= end):
            raise ValueError("shutter interval must be finite and ordered")
        return self._with(shutter_start=float(start), shutter_end=float(end))

    def with_background(self, color):
        return self._with(background_kind=abi.GT_BG_CONSTANT, background=_vec(color) + (0.0,) * 6)

    def with_vertical_gradient_background(self, nadir, horizon, zenith):
        return self._with(background_kind=abi.GT_BG_VERTICAL_GRADIENT,
                          background=_vec(nadir) + _vec(horizon) + _vec(zenith))

    def image_size(self) -> tuple[int, int, int]:
        w, h, s = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(lib().gt_camera_image_size(C.byref(self._d), C.byref(w), C.byref(h), C.byref(s)))
        return w.value, h.value, s.value

    @property
    def image_width(self) -> int:
        return self._d.image_width

    @property
    def image_height(self) -> int:
        return self.image_size()[1]

    def effective_samples_per_pixel(self) -> int:
        return self.image_size()[2]


# --------------------------------------------------------------------- images
def _gamma2_byte(c: np.ndarray) -> np.ndarray:
    """Rgb::linear_to_gamma_component then (256 * clamp(., 0, 0.999)) as u8 (colors.rs:388-422):
    the square root of the non-negative part, non-finite values as 0."""
    c = np.nan_to_num(np.asarray(c, dtype=np.float64), nan=0.0, posinf=0.0, neginf=0.0)
    g = np.sqrt(np.clip(c, 0.0, None))
    return (256.0 * np.clip(g, 0.0, 0.999)).astype(np.uint8)


def linear_color_to_rgb(color) -> tuple:
    """linear_color_to_rgb (graphics/raytracing.rs:166-168): gamma-2 display bytes."""
    return tuple(int(x) for x in _gamma2_byte(np.asarray(color, dtype=np.float64)))


TONE_MAP_NONE, TONE_MAP_REINHARD, TONE_MAP_ACES = 0, 1, 2


@dataclass(frozen=True)
class ToneMap:
    """ToneMap (graphics/display.rs:164-280): exposure, then the operator (none, Reinhard
    x / (1 + x), or the ACES fit clamped to [0, 1]) on the finite non-negative part, then
    gamma encoding (gamma 2 is the square root) and (256 * clamp(., 0, 0.999)) as u8."""

    exposure: float = 1.0
    operator: int = TONE_MAP_NONE
    gamma: float = 2.0

    def with_exposure(self, exposure: float) -> "ToneMap":
        if not (math.isfinite(exposure) and exposure >= 0.0):
            raise ValueError("tone-map exposure must be finite and non-negative")
        return ToneMap(float(exposure), self.operator, self.gamma)

    def with_operator(self, operator: int) -> "ToneMap":
        if operator not in (TONE_MAP_NONE, TONE_MAP_REINHARD, TONE_MAP_ACES):
            raise ValueError("unknown tone-mapping operator")
        return ToneMap(self.exposure, int(operator), self.gamma)

    def with_gamma(self, gamma: float) -> "ToneMap":
        if not (math.isfinite(gamma) and gamma > 0.0):
            raise ValueError("tone-map gamma must be positive and finite")
        return ToneMap(self.exposure, self.operator, float(gamma))

    def map_colors(self, c: np.ndarray) -> np.ndarray:
        """ToneMap::map_color over an array of linear colours (display.rs:262-277)."""
        v = np.asarray(c, dtype=np.float64) * self.exposure
        v = np.where(np.isfinite(v), np.maximum(v, 0.0), 0.0)
        if self.operator == TONE_MAP_REINHARD:
            v = v / (1.0 + v)
        elif self.operator == TONE_MAP_ACES:
            v = np.clip(v * (2.51 * v + 0.03) / (v * (2.43 * v + 0.59) + 0.14), 0.0, 1.0)
        if abs(self.gamma - 2.0) <= 2.220446049250313e-16:
            g = np.sqrt(v)
        else:
            with np.errstate(divide="ignore", invalid="ignore"):
                g = np.where(v <= 0.0, 0.0, np.power(np.maximum(v, 0.0), 1.0 / self.gamma))
        return (256.0 * np.clip(g, 0.0, 0.999)).astype(np.uint8)


@dataclass
class HdrImage:
    """HdrImage (graphics/display.rs:282-440): row-major linear RGB, row 0 at the top."""

    width: int
    height: int
    pixels: np.ndarray  # (H, W, 3) float32
    accepted: Optional[np.ndarray] = None
    pixels64: Optional[np.ndarray] = None

    def to_canvas(self) -> np.ndarray:
        """Gamma-2 bytes, (256 * clamp(sqrt(c), 0, 0.999)) as u8 (colors.rs:388-407)."""
        c = np.nan_to_num(self.pixels.astype(np.float64), nan=0.0)
        g = np.sqrt(np.clip(c, 0.0, None))
        return (256.0 * np.clip(g, 0.0, 0.999)).astype(np.uint8)

    def to_canvas_tone_mapped(self, tone_map: ToneMap) -> np.ndarray:
        """HdrImage::to_canvas_tone_mapped (display.rs:338-350)."""
        return tone_map.map_colors(self._linear())

    def _linear(self) -> np.ndarray:
        return self.pixels64 if self.pixels64 is not None else self.pixels.astype(np.float64)

    def pfm_bytes(self) -> bytes:
        """HdrImage::write_pfm (display.rs:365-387): little-endian f32, bottom row first,
        non-finite components written as 0."""
        c = self._linear()
        c = np.where(np.isfinite(c), c, 0.0).astype("<f4")
        return f"PF\n{self.width} {self.height}\n-1.0\n".encode() + np.ascontiguousarray(c[::-1]).tobytes()

    def radiance_hdr_bytes(self) -> bytes:
        """HdrImage::write_radiance_hdr with encode_rgbe (display.rs:394-407, 443-465): flat
        RGBE pixels in storage order (top row first)."""
        c = self._linear()
        c = np.where(np.isfinite(c), np.maximum(c, 0.0), 0.0)
        m = c.max(axis=2)
        out = np.zeros(c.shape[:2] + (4,), dtype=np.uint8)
        live = m > 1.0e-32
        with np.errstate(divide="ignore"):
            e = np.floor(np.log2(np.where(live, m, 1.0))).astype(np.int64) + 1
        scale = 256.0 * np.ldexp(1.0, -e)
        out[..., :3] = np.clip(c * scale[..., None], 0.0, 255.0).astype(np.uint8)
        out[..., 3] = np.clip(e + 128, 0, 255).astype(np.uint8)
        out[~live] = 0
        head = f"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y {self.height} +X {self.width}\n".encode()
        return head + out.tobytes()

    def save_pfm(self, path) -> None:
        """HdrImage::save_pfm (display.rs:359-363)."""
        with open(path, "wb") as f:
            f.write(self.pfm_bytes())

    def save_radiance_hdr(self, path) -> None:
        """HdrImage::save_radiance_hdr (display.rs:394-398)."""
        with open(path, "wb") as f:
            f.write(self.radiance_hdr_bytes())

    def save_extension(self, path) -> None:
        """HdrImage::save_extension (display.rs:419-431) for the HDR formats: .pfm, .hdr and
        .rgbe keep the linear data; other extensions would go through a tone-mapped canvas
        writer, which is outside this library."""
        ext = str(path).rsplit(".", 1)[-1].lower() if "." in str(path) else ""
        if ext == "pfm":
            self.save_pfm(path)
        elif ext in ("hdr", "rgbe"):
            self.save_radiance_hdr(path)
        else:
            raise ValueError("only .pfm, .hdr and .rgbe are written here")


@dataclass
class DenoisingAovs:
    """DenoisingAovs (graphics/camera.rs:491-526), linear planes."""

    beauty_linear: np.ndarray
    albedo_linear: np.ndarray
    normal_linear: np.ndarray


class Accumulator:
    """Accumulation state of one frame across renders (gt_accumulator): add samples with
    PathTracer.render_accumulate, checkpoint with save() / load()."""

    def __init__(self, width: int, height: int, precision: str = "f32", context: Optional[Context] = None):
        if precision not in ("f32", "f64"):
            raise ValueError("precision must be 'f32' or 'f64'")
        self.ctx = context or Context.default()
        self.width, self.height, self.precision = int(width), int(height), precision
        h = C.c_void_p()
        check(lib().gt_accumulator_create(self.ctx.handle, self.width, self.height,
                                          abi.GT_PRECISION_F64 if precision == "f64" else abi.GT_PRECISION_F32,
                                          C.byref(h)))
        self.h = h
        self.ctx._track(self)

    @property
    def samples(self) -> int:
        n = C.c_uint32()
        check(lib().gt_accumulator_samples(self.h, C.byref(n)))
        return int(n.value)

    def save(self) -> bytes:
        size = C.c_uint64()
        check(lib().gt_accumulator_save(self.h, None, 0, C.byref(size)))
        buf = C.create_string_buffer(size.value)
        check(lib().gt_accumulator_save(self.h, buf, size.value, C.byref(size)))
        return buf.raw

    def load(self, blob: bytes) -> None:
        check(lib().gt_accumulator_load(self.h, blob, len(blob)))

    def close(self):
        if self.h:
            lib().gt_accumulator_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------- renderer
@dataclass(frozen=True)
class RenderOptions:
    """RenderOptions (renderer.rs:20-45).  Tiles do not exist on the wavefront path;
    the tile size is accepted and ignored because the image does not depend on it."""

    tile_size: Optional[int] = None


class PathTracer:
    """PathTracer (raytracing/renderer.rs:55-875) on the GB300 wavefront integrator.

    precision: "f32" (throughput) or "f64" (the reference's arithmetic, op for op).
    schedule: "auto" (wavefront, then the persistent kernel for the last tail_slots
    pixels; 0 = the library's choice), "wavefront" or "persistent"; the image is the same.
    migrate: "default", "on" or "off": whether "auto" moves each stripe's slow pixels to a
    concurrent persistent kernel early in the frame (gt_migrate; default = on for scenes of
    at most 65,536 primitives).
    rng: "pixel" (the reference: each pixel's samples continue one random stream) or
    "substreams" (throughput mode: each sample draws from its own stream, so all of a
    pixel's samples run in parallel; the same estimator, not the same numbers)."""

    SCHEDULES = {"auto": abi.GT_SCHEDULE_AUTO, "wavefront": abi.GT_SCHEDULE_WAVEFRONT,
                 "persistent": abi.GT_SCHEDULE_PERSISTENT}
    MIGRATE = {"default": abi.GT_MIGRATE_DEFAULT, "on": abi.GT_MIGRATE_ON, "off": abi.GT_MIGRATE_OFF}
    RNG = {"pixel": abi.GT_RNG_PIXEL, "substreams": abi.GT_RNG_SUBSTREAMS}

    def __init__(self, camera: RayCamera, options: RenderOptions = RenderOptions(), precision: str = "f32",
                 context: Optional[Context] = None, profile: bool = False, schedule: str = "auto",
                 tail_slots: int = 0, stripes: int = 0, generate_blocks_per_sm: int = 0,
                 trace_blocks_per_sm: int = 0, migrate: str = "default", rng: str = "pixel"):
        if precision not in ("f32", "f64"):
            raise ValueError("precision must be 'f32' or 'f64'")
        if schedule not in self.SCHEDULES:
            raise ValueError(f"schedule must be one of {sorted(self.SCHEDULES)}")
        self.camera = camera
        self.options = options
        self.precision = precision
        self.profile = profile
        self.schedule = schedule
        self.tail_slots = int(tail_slots)
        self.stripes = int(stripes)
        self.generate_blocks_per_sm = int(generate_blocks_per_sm)
        self.trace_blocks_per_sm = int(trace_blocks_per_sm)
        if migrate not in self.MIGRATE:
            raise ValueError(f"migrate must be one of {sorted(self.MIGRATE)}")
        if rng not in self.RNG:
            raise ValueError(f"rng must be one of {sorted(self.RNG)}")
        self.migrate = migrate
        self.rng = rng
        self._ctx = context
        self.last_stats: Optional[dict] = None

    @property
    def context(self) -> Context:
        return self._ctx or Context.default()

    def _launch_kw(self) -> dict:
        return {"schedule": self.schedule, "tail_slots": self.tail_slots, "stripes": self.stripes,
                "generate_blocks_per_sm": self.generate_blocks_per_sm, "trace_blocks_per_sm": self.trace_blocks_per_sm,
                "migrate": self.migrate, "rng": self.rng}

    def with_options(self, options: RenderOptions) -> "PathTracer":
        return PathTracer(self.camera, options, self.precision, self._ctx, self.profile, **self._launch_kw())

    def _launch_opts(self, o) -> None:
        """The tracer's schedule and launch shapes into a gt_render_opts."""
        o.schedule = self.SCHEDULES[self.schedule]
        o.tail_slots = self.tail_slots
        o.stripes = self.stripes
        o.generate_blocks_per_sm = self.generate_blocks_per_sm
        o.trace_blocks_per_sm = self.trace_blocks_per_sm
        o.migrate = self.MIGRATE[self.migrate]
        o.rng = self.RNG[self.rng]

    def autotune(self, world: RayScene, lights: Optional[WeightedSamplingTargetList] = None,
                 environment: Optional[EnvironmentLight] = None, cameras=None) -> dict:
        """gt_autotune: times this tracer's frame (or the batch of `cameras`) under candidate
        stripe counts, tail sizes, wavefront blocks per SM and (schedule "auto") migration on
        or off, then (schedule "auto", or "persistent" from an earlier tune) the persistent
        schedule, and keeps the fastest in this tracer.  Launch shapes never change the image;
        migrating pixels or switching to the persistent schedule can change f32 pixels (other
        kernels fuse f32 operations differently), never f64 images or accepted counts.
        Returns {"trials", "given_ms", "best_ms", "schedule", "stripes", "tail_slots",
        "generate_blocks_per_sm", "trace_blocks_per_sm", "migrate"}."""
        ctx = self.context
        cams = list(cameras) if cameras is not None else [self.camera]
        descs = [c.desc() for c in cams]
        frames, keep = [], []
        for c in cams:
            w, h, _ = c.image_size()
            rgb = np.empty((h, w, 3), dtype=np.float32)
            f = abi.gt_frame()
            f.struct_size = C.sizeof(abi.gt_frame)
            f.width, f.height, f.device_buffers = w, h, 0
            f.rgb = rgb.ctypes.data
            frames.append(f)
            keep.append(rgb)
        jobs = (abi.gt_frame_job * len(cams))()
        for i in range(len(cams)):
            jobs[i].camera = C.pointer(descs[i])
            jobs[i].frame = C.pointer(frames[i])
        o = abi.gt_render_opts()
        o.struct_size = C.sizeof(abi.gt_render_opts)
        o.precision = abi.GT_PRECISION_F64 if self.precision == "f64" else abi.GT_PRECISION_F32
        self._launch_opts(o)
        rep = abi.gt_autotune_report()
        rep.struct_size = C.sizeof(abi.gt_autotune_report)
        sh = world._handle(ctx)
        lh = lights._handle(ctx).h if lights is not None else None
        eh = environment._handle(ctx).h if environment is not None else None
        check(lib().gt_autotune(sh.h, lh, eh, jobs, len(cams), C.byref(o), C.byref(rep)))
        self.stripes, self.tail_slots = int(o.stripes), int(o.tail_slots)
        self.generate_blocks_per_sm, self.trace_blocks_per_sm = int(o.generate_blocks_per_sm), int(o.trace_blocks_per_sm)
        self.migrate = {v: k for k, v in self.MIGRATE.items()}[int(o.migrate)]
        self.schedule = {v: k for k, v in self.SCHEDULES.items()}[int(o.schedule)]
        return {"trials": int(rep.trials), "given_ms": float(rep.given_ms), "best_ms": float(rep.best_ms),
                **self._launch_kw()}

    def render_accumulate(self, world: RayScene, accumulator: Accumulator, samples: int,
                          lights: Optional[WeightedSamplingTargetList] = None,
                          environment: Optional[EnvironmentLight] = None) -> HdrImage:
        """Adds `samples` samples per pixel to `accumulator` with this tracer's camera
        (random sampling, no adaptive stopping) and returns the image of everything
        accumulated so far (gt_render_accumulate)."""
        ctx = accumulator.ctx
        w, h, _ = self.camera.image_size()
        want64 = accumulator.precision == "f64"
        img = HdrImage(w, h, np.empty((h, w, 3), dtype=np.float32), np.empty((h, w), dtype=np.uint32),
                       np.empty((h, w, 3), dtype=np.float64) if want64 else None)
        f = abi.gt_frame()
        f.struct_size = C.sizeof(abi.gt_frame)
        f.width, f.height, f.device_buffers = w, h, 0
        f.rgb = img.pixels.ctypes.data
        f.accepted = img.accepted.ctypes.data
        f.rgb64 = img.pixels64.ctypes.data if want64 else None
        o = abi.gt_render_opts()
        o.struct_size = C.sizeof(abi.gt_render_opts)
        o.profile = 1 if self.profile else 0
        self._launch_opts(o)
        if self.schedule == "persistent":  # accumulation runs on the wavefront
            o.schedule = abi.GT_SCHEDULE_AUTO
        stats = abi.gt_render_stats()
        o.stats = C.pointer(stats)
        sh = world._handle(ctx)
        lh = lights._handle(ctx).h if lights is not None else None
        eh = environment._handle(ctx).h if environment is not None else None
        check(lib().gt_render_accumulate(sh.h, lh, eh, C.byref(self.camera.desc()), int(samples), accumulator.h,
                                         C.byref(o), C.byref(f)))
        self.last_stats = stats.as_dict()
        return img

    def render_batch_hdr_images(self, world: RayScene, cameras, lights: Optional[WeightedSamplingTargetList] = None,
                                environment: Optional[EnvironmentLight] = None, want64: bool = False) -> list:
        """One image per camera, all rendered together (gt_render_batch): the per-frame loop
        around render_with_*_hdr_image for an animation or a camera sweep.  This tracer's
        camera is not used; each frame is rendered with its own.  In f32, frames of one
        width run through the striped wavefront as one image of their rows (schedule
        "auto" or "wavefront"); otherwise all pixels go through one persistent launch."""
        ctx = self.context
        cams = list(cameras)
        descs = [c.desc() for c in cams]
        frames, images = [], []
        for c in cams:
            w, h, _ = c.image_size()
            img = HdrImage(w, h, np.empty((h, w, 3), dtype=np.float32), np.empty((h, w), dtype=np.uint32),
                           np.empty((h, w, 3), dtype=np.float64) if want64 else None)
            f = abi.gt_frame()
            f.struct_size = C.sizeof(abi.gt_frame)
            f.width, f.height, f.device_buffers = w, h, 0
            f.rgb = img.pixels.ctypes.data
            f.accepted = img.accepted.ctypes.data
            f.rgb64 = img.pixels64.ctypes.data if want64 else None
            frames.append(f)
            images.append(img)
        jobs = (abi.gt_frame_job * len(cams))()
        for i in range(len(cams)):
            jobs[i].camera = C.pointer(descs[i])
            jobs[i].frame = C.pointer(frames[i])
        o = abi.gt_render_opts()
        o.struct_size = C.sizeof(abi.gt_render_opts)
        o.precision = abi.GT_PRECISION_F64 if self.precision == "f64" else abi.GT_PRECISION_F32
        o.profile = 1 if self.profile else 0
        self._launch_opts(o)
        stats = abi.gt_render_stats()
        o.stats = C.pointer(stats)
        sh = world._handle(ctx)
        lh = lights._handle(ctx).h if lights is not None else None
        eh = environment._handle(ctx).h if environment is not None else None
        check(lib().gt_render_batch(sh.h, lh, eh, jobs, len(cams), C.byref(o)))
        self.last_stats = stats.as_dict()
        return images

    def render_progressive(self, world: RayScene, progress, lights: Optional[WeightedSamplingTargetList] = None,
                           environment: Optional[EnvironmentLight] = None) -> HdrImage:
        """PathTracer::render_progressive (renderer.rs:136-146): `progress(update)` is called
        while the frame renders with update.completed / update.total (samples) and
        update.pixels, the image as far as it is known (finished pixels final, the rest 0).
        An exception raised by `progress` stops the render and is re-raised, as the
        reference returns the callback's first error."""
        w, h, _ = self.camera.image_size()
        preview = np.zeros((h, w, 3), dtype=np.float32)
        raised: list = []

        class Update:
            def __init__(self, completed, total):
                self.completed, self.total, self.pixels = int(completed), int(total), preview

        @abi.GT_PROGRESS_FN
        def cb(user, done, total):
            try:
                progress(Update(done, total))
                return 0
            except BaseException as exc:  # handed back to the caller after the cancel
                raised.append(exc)
                return 1

        try:
            return self._render(world, lights, environment, progress_fn=cb, progress_rgb=preview)
        except GartusError:
            if raised:
                raise raised[0]
            raise

    def _render(self, world: RayScene, lights: Optional[WeightedSamplingTargetList],
                environment: Optional[EnvironmentLight], aovs: bool = False, want64: bool = False,
                progress_fn=None, progress_rgb: Optional[np.ndarray] = None):
        ctx = self.context
        w, h, _ = self.camera.image_size()
        rgb = np.empty((h, w, 3), dtype=np.float32)
        acc = np.empty((h, w), dtype=np.uint32)
        rgb64 = np.empty((h, w, 3), dtype=np.float64) if want64 else None
        alb = np.empty((h, w, 3), dtype=np.float32) if aovs else None
        nrm = np.empty((h, w, 3), dtype=np.float32) if aovs else None
        f = abi.gt_frame()
        f.struct_size = C.sizeof(abi.gt_frame)
        f.width, f.height, f.device_buffers = w, h, 0
        f.rgb = rgb.ctypes.data
        f.accepted = acc.ctypes.data
        f.rgb64 = rgb64.ctypes.data if want64 else None
        f.albedo = alb.ctypes.data if aovs else None
        f.normal = nrm.ctypes.data if aovs else None
        o = abi.gt_render_opts()
        o.struct_size = C.sizeof(abi.gt_render_opts)
        o.precision = abi.GT_PRECISION_F64 if self.precision == "f64" else abi.GT_PRECISION_F32
        o.aovs = 1 if aovs else 0
        o.profile = 1 if self.profile else 0
        self._launch_opts(o)
        if progress_fn is not None:
            o.progress = progress_fn
            o.progress_rgb = progress_rgb.ctypes.data if progress_rgb is not None else None
        stats = abi.gt_render_stats()
        o.stats = C.pointer(stats)
        sh = world._handle(ctx)
        lh = lights._handle(ctx).h if lights is not None else None
        eh = environment._handle(ctx).h if environment is not None else None
        check(lib().gt_render(sh.h, lh, eh, C.byref(self.camera.desc()), C.byref(o), C.byref(f)))
        self.last_stats = stats.as_dict()
        img = HdrImage(w, h, rgb, acc, rgb64)
        if aovs:
            return img, alb, nrm
        return img

    # render / render_hdr_image (renderer.rs:101-117)
    def render_hdr_image(self, world: RayScene, want64: bool = False) -> HdrImage:
        return self._render(world, None, None, want64=want64)

    def render(self, world: RayScene) -> np.ndarray:
        return self.render_hdr_image(world).to_canvas()

    # render_ray_scene_hdr_image (renderer.rs:193-200)
    def render_ray_scene_hdr_image(self, scene: RayScene, want64: bool = False) -> HdrImage:
        lights = scene.emissive_targets()
        if lights.is_empty():
            return self.render_hdr_image(scene, want64)
        return self.render_with_lights_hdr_image(scene, lights, want64)

    def render_ray_scene(self, scene: RayScene) -> np.ndarray:
        return self.render_ray_scene_hdr_image(scene).to_canvas()

    # render_with_lights_hdr_image (renderer.rs:391-406)
    def render_with_lights_hdr_image(self, world: RayScene, lights: WeightedSamplingTargetList,
                                     want64: bool = False) -> HdrImage:
        return self._render(world, lights, None, want64=want64)

    def render_with_lights(self, world, lights) -> np.ndarray:
        return self.render_with_lights_hdr_image(world, lights).to_canvas()

    # render_with_light_connections (renderer.rs:771-786): forces NEE
    def render_with_light_connections_hdr_image(self, world, lights, want64: bool = False) -> HdrImage:
        cam = self.camera.with_direct_lighting_mode(abi.GT_DIRECT_NEXT_EVENT_ESTIMATION)
        return PathTracer(cam, self.options, self.precision, self._ctx, self.profile, **self._launch_kw())._render(
            world, lights, None, want64=want64)

    # render_with_environment_hdr_image (renderer.rs:431-449)
    def render_with_environment_hdr_image(self, world: RayScene, environment: EnvironmentLight,
                                          want64: bool = False) -> HdrImage:
        return self._render(world, None, environment, want64=want64)

    def render_with_environment(self, world, environment) -> np.ndarray:
        return self.render_with_environment_hdr_image(world, environment).to_canvas()

    # render_with_lights_and_environment_hdr_image (renderer.rs:588-609)
    def render_with_lights_and_environment_hdr_image(self, world, lights, environment,
                                                     want64: bool = False) -> HdrImage:
        return self._render(world, lights, environment, want64=want64)

    # render_denoising_aovs (renderer.rs:121-129) and render_ray_scene_denoising_aovs (217-224)
    def render_denoising_aovs(self, world: RayScene) -> DenoisingAovs:
        img, alb, nrm = self._render(world, None, None, aovs=True)
        return DenoisingAovs(img.pixels, alb, nrm)

    def render_ray_scene_denoising_aovs(self, scene: RayScene) -> DenoisingAovs:
        lights = scene.emissive_targets()
        img, alb, nrm = self._render(scene, None if lights.is_empty() else lights, None, aovs=True)
        return DenoisingAovs(img.pixels, alb, nrm)

    # render_ray_scene_with_light_connections (raytracing.rs:1748-1776): the scene's emissive
    # targets as light connections
    def render_ray_scene_with_light_connections_hdr_image(self, scene: RayScene, want64: bool = False) -> HdrImage:
        return self.render_with_light_connections_hdr_image(scene, scene.emissive_targets(), want64=want64)

    def render_tone_mapped(self, world: RayScene, tone_map: "ToneMap") -> np.ndarray:
        """render_tone_mapped (renderer.rs:101-117 with ToneMap, display.rs:338-350)."""
        return self.render_hdr_image(world).to_canvas_tone_mapped(tone_map)

    # render_scene / render_scene_hdr_image / render_scene_denoising_aovs /
    # render_scene_with_lights / render_scene_with_light_connections (renderer.rs:309-371):
    # the surface scene compiled to a RayScene (Lambertian policy) on every call
    def render_scene_hdr_image(self, scene: "SurfaceScene", want64: bool = False) -> HdrImage:
        return self.render_hdr_image(scene.to_ray_scene(), want64=want64)

    def render_scene(self, scene: "SurfaceScene") -> np.ndarray:
        return self.render_scene_hdr_image(scene).to_canvas()

    def render_scene_denoising_aovs(self, scene: "SurfaceScene") -> DenoisingAovs:
        return self.render_denoising_aovs(scene.to_ray_scene())

    def render_scene_with_lights(self, scene: "SurfaceScene", lights) -> np.ndarray:
        return self.render_with_lights(scene.to_ray_scene(), lights)

    def render_scene_with_light_connections_hdr_image(self, scene: "SurfaceScene", lights,
                                                       want64: bool = False) -> HdrImage:
        return self.render_with_light_connections_hdr_image(scene.to_ray_scene(), lights, want64=want64)

    def trace_primary(self, scene: RayScene, stride: int = 1):
        """Primary probe rays (ray_for_pixel) through the f64 reference-layout BVH:
        (prim_ids, t, BvhTraversalStats) (benches/render_performance.rs:42-93)."""
        w, h, _ = self.camera.image_size()
        stride = max(int(stride), 1)
        n = ((w + stride - 1) // stride) * ((h + stride - 1) // stride)
        ids = np.empty(n, dtype=np.int32)
        t = np.empty(n, dtype=np.float64)
        st = abi.gt_bvh_stats()
        check(lib().gt_trace_primary(scene._handle(self.context).h, C.byref(self.camera.desc()), stride,
                                     ids.ctypes.data_as(C.c_void_p), t.ctypes.data_as(C.c_void_p), C.byref(st)))
        return ids, t, st.as_dict()

    def trace_primary_f32(self, scene: RayScene, stride: int = 1):
        """The same probe rays through the renderer's f32 walk with near ties re-traced in
        f64 (gt_trace_primary_f32): (prim_ids, t, refined, report)."""
        w, h, _ = self.camera.image_size()
        stride = max(int(stride), 1)
        n = ((w + stride - 1) // stride) * ((h + stride - 1) // stride)
        ids = np.empty(n, dtype=np.int32)
        t = np.empty(n, dtype=np.float64)
        refined = np.empty(n, dtype=np.uint8)
        rep = abi.gt_trace_report()
        rep.struct_size = C.sizeof(abi.gt_trace_report)
        check(lib().gt_trace_primary_f32(scene._handle(self.context).h, C.byref(self.camera.desc()), stride,
                                         ids.ctypes.data_as(C.c_void_p), t.ctypes.data_as(C.c_void_p),
                                         refined.ctypes.data_as(C.c_void_p), C.byref(rep)))
        return ids, t, refined, rep.as_dict()


# ------------------------------------------------------------ surface scenes
@dataclass(frozen=True)
class SurfaceMaterial:
    """SurfaceMaterial (graphics/material.rs:12-110): the renderer-neutral colours and the
    optional refractive index that the ray materials are derived from."""

    ambient_color: tuple = (0.1, 0.1, 0.1)
    base_color: tuple = (0.5, 0.5, 0.5)
    specular_color: tuple = (0.9, 0.9, 0.9)
    shininess: float = 200.0
    refractive_index: Optional[float] = None

    def __post_init__(self):
        vals = list(self.ambient_color) + list(self.base_color) + list(self.specular_color) + [self.shininess]
        if not all(math.isfinite(float(x)) for x in vals):  # SurfaceMaterial::new asserts finite values
            raise ValueError("surface material colours and shininess must be finite")
        if self.refractive_index is not None and not (math.isfinite(self.refractive_index) and
                                                      self.refractive_index > 0.0):
            raise ValueError("refractive index must be positive and finite")  # lighting.rs:268-273

    # SurfaceMaterial::as_* (raytracing/material.rs:2238-2262)
    def as_lambertian(self) -> RayMaterial:
        return RayMaterial.lambertian(self.base_color)

    def as_metal(self, fuzz: float) -> RayMaterial:
        return RayMaterial.metal(self.specular_color, fuzz)

    def as_ggx_microfacet(self, roughness: float) -> RayMaterial:
        return RayMaterial.ggx_microfacet(self.specular_color, roughness)

    def as_dielectric(self) -> Optional[RayMaterial]:
        return None if self.refractive_index is None else RayMaterial.dielectric(self.refractive_index)


class SurfaceRayMaterialMode:
    """SurfaceRayMaterialMode (raytracing/scene.rs:30-72): Lambertian (the default),
    PreferDielectric, PreferMetal{fuzz} or Custom(mapper)."""

    def __init__(self, kind: str, fuzz: float = 0.0, mapper=None):
        if kind not in ("lambertian", "prefer_dielectric", "prefer_metal", "custom"):
            raise ValueError("unknown surface material mode")
        if kind == "custom" and mapper is None:
            raise ValueError("a custom mode needs a mapper")
        self.kind, self.fuzz, self.mapper = kind, float(fuzz), mapper

    @classmethod
    def lambertian(cls) -> "SurfaceRayMaterialMode":
        return cls("lambertian")

    @classmethod
    def prefer_dielectric(cls) -> "SurfaceRayMaterialMode":
        return cls("prefer_dielectric")

    @classmethod
    def prefer_metal(cls, fuzz: float) -> "SurfaceRayMaterialMode":
        return cls("prefer_metal", fuzz=fuzz)

    @classmethod
    def custom(cls, mapper) -> "SurfaceRayMaterialMode":
        return cls("custom", mapper=mapper)

    def convert(self, material: SurfaceMaterial) -> RayMaterial:
        """SurfaceRayMaterialMode::convert (scene.rs:56-67)."""
        if self.kind == "lambertian":
            return material.as_lambertian()
        if self.kind == "prefer_dielectric":
            d = material.as_dielectric()
            return d if d is not None else material.as_lambertian()
        if self.kind == "prefer_metal":
            return material.as_metal(self.fuzz)
        out = self.mapper(material)
        if not isinstance(out, RayMaterial):
            raise TypeError("a custom surface material mapper must return a RayMaterial")
        return out


@dataclass
class SurfaceMesh:
    """SurfaceMesh (graphics/scene.rs:17-60): triangles plus a surface material."""

    triangles: np.ndarray  # (N, 3, 3)
    material: SurfaceMaterial = field(default_factory=SurfaceMaterial)

    @property
    def base_color(self) -> tuple:
        return self.material.base_color


@dataclass
class SurfaceScene:
    """SurfaceScene (graphics/scene.rs) restricted to what to_ray_scene consumes."""

    meshes: list = field(default_factory=list)

    def add_mesh(self, triangles: np.ndarray, base_color=(0.5, 0.5, 0.5),
                 material: Optional[SurfaceMaterial] = None) -> None:
        mat = material if material is not None else SurfaceMaterial(base_color=_vec(base_color))
        self.meshes.append(SurfaceMesh(np.asarray(triangles, dtype=np.float64).reshape(-1, 3, 3), mat))

    def __len__(self) -> int:
        return len(self.meshes)

    def to_ray_scene(self, leaf_size: int = 4) -> RayScene:
        """SurfaceScene::to_ray_scene (scene.rs:1606-1608): the Lambertian mode."""
        return self.to_ray_scene_with_material_mode(SurfaceRayMaterialMode.lambertian(), leaf_size)

    def to_ray_scene_with_material_mode(self, mode: SurfaceRayMaterialMode, leaf_size: int = 4) -> RayScene:
        """RayScene::from_surface_scene_with_material_mode_and_bvh_options (scene.rs:1517-1547):
        one material per mesh through `mode`, the meshes' triangles in order, BVH built."""
        scene = RayScene()
        for mesh in self.meshes:
            mid = scene.add_material(mode.convert(mesh.material))
            scene.add_triangles_array(mid, mesh.triangles)
        scene.build_bvh_with_options(leaf_size)
        return scene
