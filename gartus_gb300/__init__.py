"""gartus_gb300 — a GB300 (sm_103a) wavefront path tracer that drops in for gartus's
`PathTracer` render path over a compiled `RayScene`.

The compute lives in libgartus_gpu.so (C ABI: include/gartus_gpu.h); this package is the
host-side mirror of the reference's Rust API over that ABI.
"""
from . import abi
from ._lib import GartusError, lib
from .raytracing import (
    GLASS, INFINITY, SHADOW_ACNE_EPSILON, WIDESCREEN_ASPECT_RATIO, Context, DenoisingAovs,
    EnvironmentLight, HdrImage, PathTracer, RayCamera, RayGeometry, RayMaterial, RayScene,
    RenderOptions, SamplingTargetList, SurfaceMesh, SurfaceScene, WeightedSamplingTargetList,
)

__all__ = [
    "abi", "lib", "GartusError", "GLASS", "INFINITY", "SHADOW_ACNE_EPSILON", "WIDESCREEN_ASPECT_RATIO",
    "Context", "DenoisingAovs", "EnvironmentLight", "HdrImage", "PathTracer", "RayCamera", "RayGeometry",
    "RayMaterial", "RayScene", "RenderOptions", "SamplingTargetList", "SurfaceMesh", "SurfaceScene",
    "WeightedSamplingTargetList",
]
