"""Check 2's divergence classifier: why an f32 pixel differs from the reference.

The f32 GPU path draws the reference's random numbers in the reference's order, so a
pixel can leave the f64 result by more than the tolerance only where f32 rounding changed a
discrete decision of one of its samples (which primitive a ray hits, the Schlick or total
internal reflection choice, Russian roulette, the light/material mixture choice, a pdf
cut-off, a shadow test, a checker cell, an environment texel, the adaptive stop test) or
where a long chain of f32 operations drifted.  For each such pixel the oracle renders the pixel twice, in f64
and in f32, recording every decision in order (oracle.OracleScene.pixel_trace); the first
decision whose outcome differs between the two runs is the cause.  When no decision
differs but the f32 oracle also leaves the f64 result, the cause is continuous f32
rounding.  When the f32 oracle stays with f64, the GPU's own f32 rounding (fused
multiply-adds, CUDA's division, square root and transcendentals) moved the pixel; the
cause is then the first decision of the f64 run that lies within NEAR of its boundary,
or, with none, the GPU's continuous drift where the pixel stays within GPU_DRIFT of f64
(for at most GPU_DRIFT_SHARE of the image).  Anything else is unexplained, and the parity
tests allow no unexplained pixel.
"""
from __future__ import annotations

from collections import Counter

import numpy as np

import oracle
from tests.helpers import rel_err

CAUSES = {
    1: "sample dropped (non-finite)",
    2: "closest hit (edge, silhouette or near tie)",
    3: "material scatter (absorbed / below-surface direction)",
    4: "dielectric (Schlick draw or total internal reflection)",
    5: "Russian roulette draw",
    6: "light/material mixture draw",
    7: "pdf cut-off",
    8: "area-light shadow ray",
    9: "environment shadow ray",
    10: "light target pick",
    11: "checker texture cell",
    12: "environment texel pick",
    14: "adaptive stop test",
}
CONTINUOUS = "continuous f32 rounding (no decision flips; the f32 oracle drifts too)"
GPU_ROUNDING = "continuous GPU f32 rounding (within 1e-3; fused multiply-adds, approximate division)"
UNEXPLAINED = "unexplained"
# Decisions whose f64 margin the trace records (0 at the boundary): a hit's grazing cosine
# or edge distance, the Schlick / total-internal-reflection margin, the draws of Russian
# roulette, the mixture and the light pick, the shadow hits' margins, a checker cell's
# boundary distance, the environment CDF step, the adaptive error estimate's distance to
# its threshold.
MARGIN_TYPES = (2, 4, 5, 6, 8, 9, 10, 11, 12, 14)
NEAR = 1e-3
# The GPU's f32 kernels contract multiply-adds and use the hardware's approximate division
# and square root (within 2 ulp), which the f32 oracle does not; over a long path their
# drift can pass the tolerance where the oracle's stays below it.  A pixel with no decision
# flipped or near its boundary that stays within GPU_DRIFT (relative, floor 1e-3) of f64 is
# attributed to that drift; at most GPU_DRIFT_SHARE of an image's pixels may be.
GPU_DRIFT = 1e-3
GPU_DRIFT_SHARE = 0.005


def divergent_pixels(x, ref, tol=1e-4):
    """Pixels of x more than tol (relative, floor 1e-3) from ref in some channel."""
    return rel_err(x, ref, floor=1e-3).max(axis=2) > tol


def first_flip(t64, t32):
    """Index of the first decision whose (type, outcome) differs between the two traces,
    or None when they agree throughout."""
    (a_t, a_o, _), (b_t, b_o, _) = t64, t32
    n = min(len(a_t), len(b_t))
    same = (a_t[:n] == b_t[:n]) & (a_o[:n] == b_o[:n])
    bad = np.flatnonzero(~same)
    if bad.size:
        return int(bad[0])
    return None if len(a_t) == len(b_t) else n


def classify(scene, cam, x32, ref64, ref32, lights=None, env=None, tol=1e-4, limit=None, rng="pixel"):
    """Causes of the pixels where the f32 image x32 leaves the f64 reference ref64 by more
    than tol: a Counter of cause names and a list of (y, x, cause, margin) entries, where
    margin is the f64 run's margin of the attributed decision where it has one (for an
    unexplained pixel: the three values and the decision nearest its boundary)."""
    o = oracle.OracleScene.from_ray_scene(scene)
    la = lights.to_array() if lights is not None else None
    div = divergent_pixels(x32, ref64, tol)
    counts, rows = Counter(), []
    for y, x in np.argwhere(div)[:limit]:
        t64 = o.pixel_trace(cam.desc(), int(x), int(y), la, env, precision=1, rng=rng)
        t32 = o.pixel_trace(cam.desc(), int(x), int(y), la, env, precision=0, rng=rng)
        k = first_flip(t64, t32)
        margin = None
        if k is not None:
            types = t64[0] if k < len(t64[0]) else t32[0]
            cause = CAUSES.get(int(types[k]), f"decision type {int(types[k])}")
            if k < len(t64[0]) and int(t64[0][k]) in MARGIN_TYPES:
                margin = float(t64[2][k])
        elif rel_err(ref32[y, x], ref64[y, x], floor=1e-3).max() > tol:
            cause = CONTINUOUS
        else:
            near = np.flatnonzero(np.isin(t64[0], MARGIN_TYPES) & (np.abs(t64[2]) < NEAR))
            if near.size:
                j = int(near[0])
                cause = "near-boundary " + CAUSES.get(int(t64[0][j]), str(int(t64[0][j])))
                margin = float(t64[2][j])
            elif rel_err(x32[y, x], ref64[y, x], floor=1e-3).max() <= GPU_DRIFT:
                cause = GPU_ROUNDING
            else:
                cause = UNEXPLAINED
                m = np.flatnonzero(np.isin(t64[0], MARGIN_TYPES))
                j = int(m[np.argmin(np.abs(t64[2][m]))]) if m.size else -1
                margin = {"gpu": x32[y, x].tolist(), "f64": ref64[y, x].tolist(), "f32": ref32[y, x].tolist(),
                          "decisions": len(t64[0]), "nearest": (CAUSES.get(int(t64[0][j]), int(t64[0][j])),
                                                                float(t64[2][j])) if j >= 0 else None}
        counts[cause] += 1
        rows.append((int(y), int(x), cause, margin))
    return counts, rows


def report(name, counts, total):
    n = sum(counts.values())
    parts = ", ".join(f"{c}: {k}" for c, k in counts.most_common())
    print(f"{name}: {n}/{total} pixels beyond 1e-4 of f64 — {parts if parts else 'none'}")


def assert_explained(name, scene, cam, x32, ref64, ref32, lights=None, env=None, tol=1e-4, rng="pixel"):
    """Classifies the f32 image's divergent pixels, prints the counts by cause, and fails
    on any unexplained pixel (zero slack).  Returns the Counter.  rng: the per-sample
    streams the images were rendered with ("pixel" or "substreams")."""
    counts, rows = classify(scene, cam, x32, ref64, ref32, lights, env, tol, rng=rng)
    report(name, counts, ref64.shape[0] * ref64.shape[1])
    bad = [r for r in rows if r[2] == UNEXPLAINED]
    assert not bad, f"{name}: {len(bad)} unexplained divergent pixels, first {bad[:5]}"
    total = ref64.shape[0] * ref64.shape[1]
    assert counts[GPU_ROUNDING] <= max(1, GPU_DRIFT_SHARE * total), \
        f"{name}: {counts[GPU_ROUNDING]} pixels drift beyond 1e-4 without a decision near its boundary"
    return counts


def assert_modes_agree(name, scene, cam, a, b, lights=None, env=None, tol=1e-4, rng="pixel"):
    """Two f32 renders of one frame by different kernels (a batch and a single frame,
    accumulated chunks and one render, another schedule): every pixel where they differ
    must be a pixel where one of them leaves the f64 reference for an explained cause."""
    o = oracle.OracleScene.from_ray_scene(scene)
    la = lights.to_array() if lights is not None else None
    ref64, _ = o.render(cam.desc(), la, env, precision=1, threads=8, rng=rng)
    ref32, _ = o.render(cam.desc(), la, env, precision=0, threads=8, rng=rng)
    assert_explained(f"{name} (a)", scene, cam, a, ref64, ref32, lights, env, tol, rng=rng)
    assert_explained(f"{name} (b)", scene, cam, b, ref64, ref32, lights, env, tol, rng=rng)
    differ = divergent_pixels(a, np.asarray(b, dtype=np.float64), tol)
    covered = divergent_pixels(a, ref64, tol) | divergent_pixels(b, ref64, tol)
    assert not (differ & ~covered).any(), f"{name}: {int((differ & ~covered).sum())} pixels differ between the " \
                                          "two renders while both agree with f64"
