"""The learned denoiser (gt_denoiser_*, gt_denoise) over the AOVs of
PathTracer.render_denoising_aovs (raytracing/renderer.rs:121-129; DenoisingAovs,
graphics/camera.rs:491-526).

The reference stops at the AOVs; this module adds the network that consumes them:

* `Denoiser` wraps a gt_denoiser: a 5-level U-Net (32/48/64/80/96 channels) whose
  convolutions run as BF16 tensor-core kernels accumulating in FP32, trained on the GPU by
  the library's own forward and backward kernels (`train_step`) and applied with the
  split-buffer per-tile fallback to the plain render (`denoise`).
* `training_scene` / `render_training_set` render low-sample / high-sample pairs with this
  package's own path tracer; `train` runs the optimisation loop over random crops.

Training tensors live on the device (torch CUDA tensors are the containers); `denoise`
accepts host numpy arrays or device tensors.
"""
from __future__ import annotations

import ctypes as C
import math
import struct
import time
from dataclasses import dataclass
from pathlib import Path
from typing import Optional

import numpy as np

from . import abi
from ._lib import check, lib
from .raytracing import (
    GLASS, Accumulator, Context, EnvironmentLight, PathTracer, RayCamera, RayMaterial, RayScene,
    SamplingTargetList,
)
from . import scenes

# (cin, cout, relu) per layer, in the flat parameter order of gt_denoiser_get_params.
CHANNELS = (32, 48, 64, 80, 96)


def layer_shapes() -> list:
    c = CHANNELS
    shapes = [(9, c[0], True), (c[0], c[0], True)]
    for lv in range(1, len(c)):
        shapes += [(c[lv - 1], c[lv], True), (c[lv], c[lv], True)]
    for lv in range(len(c) - 2, -1, -1):
        shapes += [(c[lv + 1] + c[lv], c[lv], True), (c[lv], c[lv], True)]
    shapes.append((c[0], 3, False))
    return shapes


def param_count() -> int:
    return sum(cout * 9 * cin + cout for cin, cout, _ in layer_shapes())


WEIGHTS_MAGIC = b"GTDN0001"
DEFAULT_WEIGHTS = Path(__file__).resolve().parent / "weights" / "denoiser_unet.bin"


def _device_ptr(t, shape_tail=(3,), name="tensor") -> int:
    import torch

    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != torch.float32 or not t.is_contiguous():
        raise TypeError(f"{name} must be a contiguous float32 tensor")
    if tuple(t.shape[-len(shape_tail):]) != tuple(shape_tail):
        raise ValueError(f"{name} must end in {shape_tail}")
    return t.data_ptr()


class Denoiser:
    """gt_denoiser: the network, its FP32 master weights and its Adam state."""

    def __init__(self, seed: int = 0, context: Optional[Context] = None):
        self.ctx = context or Context.default()
        h = C.c_void_p()
        check(lib().gt_denoiser_create(self.ctx.handle, int(seed) & (2**64 - 1), C.byref(h)))
        self.h = h
        self.ctx._track(self)
        n = C.c_uint64()
        check(lib().gt_denoiser_param_count(self.h, C.byref(n)))
        self.param_count = int(n.value)

    # -- parameters
    def get_params(self) -> np.ndarray:
        out = np.empty(self.param_count, dtype=np.float32)
        check(lib().gt_denoiser_get_params(self.h, out.ctypes.data, self.param_count))
        return out

    def set_params(self, params) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32).ravel()
        check(lib().gt_denoiser_set_params(self.h, p.ctypes.data, p.size))

    def save(self, path) -> None:
        p = self.get_params()
        with open(path, "wb") as f:
            f.write(WEIGHTS_MAGIC + struct.pack("<Q", p.size) + p.astype("<f4").tobytes())

    def load(self, path) -> None:
        raw = Path(path).read_bytes()
        if raw[:8] != WEIGHTS_MAGIC:
            raise ValueError(f"{path} is not a denoiser weight file")
        (n,) = struct.unpack("<Q", raw[8:16])
        if n != self.param_count or len(raw) != 16 + 4 * n:
            raise ValueError(f"{path} holds {n} parameters; the network has {self.param_count}")
        self.set_params(np.frombuffer(raw[16:], dtype="<f4"))

    @classmethod
    def pretrained(cls, path=DEFAULT_WEIGHTS, context: Optional[Context] = None) -> "Denoiser":
        d = cls(0, context)
        d.load(path)
        return d

    # -- training
    def train_step(self, beauty, target, albedo=None, normal=None, lr: float = 1e-3, want_grad: bool = False):
        """One step on a device batch [n, h, w, 3] (h, w multiples of 16).  Returns the L1
        loss on log(1 + x) before the step, and with want_grad the flat gradient."""
        n, h, w = (int(s) for s in beauty.shape[:3])
        ptrs = [_device_ptr(beauty, name="beauty"), _device_ptr(target, name="target")]
        for t, name in ((albedo, "albedo"), (normal, "normal")):
            if t is not None and tuple(t.shape) != tuple(beauty.shape):
                raise ValueError(f"{name} must have the beauty image's shape")
        if tuple(target.shape) != tuple(beauty.shape):
            raise ValueError("target must have the beauty image's shape")
        a = _device_ptr(albedo, name="albedo") if albedo is not None else None
        nn = _device_ptr(normal, name="normal") if normal is not None else None
        loss = C.c_float()
        grad = np.empty(self.param_count, dtype=np.float32) if want_grad else None
        check(lib().gt_denoiser_train_step(self.h, ptrs[0], a, nn, ptrs[1], n, h, w, float(lr), C.byref(loss),
                                           grad.ctypes.data if want_grad else None))
        return (float(loss.value), grad) if want_grad else float(loss.value)

    # -- inference
    def denoise(self, beauty, albedo=None, normal=None, beauty_half=None, tile: int = 16, threshold: float = 3.0):
        """Denoises one [h, w, 3] frame.  Host numpy arrays give a numpy result, CUDA tensors
        a CUDA tensor.  With beauty_half (the mean of the first half of the same samples)
        each tile whose split-buffer residual test fails keeps the plain render; returns
        (image, per-tile fallback flags or None)."""
        import_torch = not isinstance(beauty, np.ndarray)
        h, w = int(beauty.shape[0]), int(beauty.shape[1])
        inp = abi.gt_denoise_input()
        inp.struct_size = C.sizeof(abi.gt_denoise_input)
        inp.width, inp.height = w, h
        keep = []
        if import_torch:
            import torch

            inp.device_buffers = 1
            out = torch.empty((h, w, 3), dtype=torch.float32, device=beauty.device)

            def ptr(t, name):
                if t is None:
                    return None
                if tuple(t.shape) != (h, w, 3):
                    raise ValueError(f"{name} must be [h, w, 3]")
                return _device_ptr(t, name=name)
            out_ptr = out.data_ptr()
        else:
            inp.device_buffers = 0
            out = np.empty((h, w, 3), dtype=np.float32)

            def ptr(a, name):
                if a is None:
                    return None
                a = np.ascontiguousarray(a, dtype=np.float32)
                if a.shape != (h, w, 3):
                    raise ValueError(f"{name} must be [h, w, 3]")
                keep.append(a)
                return a.ctypes.data
            out_ptr = out.ctypes.data
        inp.beauty = ptr(beauty, "beauty")
        inp.beauty_half = ptr(beauty_half, "beauty_half")
        inp.albedo = ptr(albedo, "albedo")
        inp.normal = ptr(normal, "normal")
        t = int(tile) if tile else 16
        flags = np.zeros(((h + t - 1) // t) * ((w + t - 1) // t), dtype=np.uint8)
        count = C.c_uint32()
        check(lib().gt_denoise(self.h, C.byref(inp), t, float(threshold), out_ptr, flags.ctypes.data,
                               C.byref(count)))
        return out, (flags.reshape((h + t - 1) // t, (w + t - 1) // t) if beauty_half is not None else None)

    def close(self):
        if getattr(self, "h", None):
            lib().gt_denoiser_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------- training data
def _sky(rng: scenes.SampleRng, width: int = 256, height: int = 128) -> np.ndarray:
    el = rng.random_range(10.0, 70.0)
    az = rng.random_range(0.0, 360.0)
    return scenes.sky_with_sun(width, height, el, az, 2.0, rng.random_range(1.0, 100.0) * 20.0)


def _random_material(rng: scenes.SampleRng) -> RayMaterial:
    u = rng.random_double()
    col = (rng.random_range(0.1, 0.9), rng.random_range(0.1, 0.9), rng.random_range(0.1, 0.9))
    if u < 0.5:
        return RayMaterial.lambertian(col)
    if u < 0.75:
        return RayMaterial.ggx_microfacet(col, rng.random_range(0.05, 0.6))
    if u < 0.9:
        return RayMaterial.metal(col, rng.random_range(0.0, 0.5))
    return RayMaterial.dielectric(GLASS)


@dataclass
class TrainingScene:
    scene: RayScene
    camera: RayCamera
    lights: Optional[SamplingTargetList] = None
    environment: Optional[EnvironmentLight] = None


def training_scene(seed: int, size: int = 256) -> TrainingScene:
    """One seeded random scene from three families: a field of spheres under a sky
    gradient (the final-scene generator), a box room with a ceiling light and random
    objects (the Cornell generator), or a small Perlin height field with tori under an
    HDR sky with a sun (the mesh generator).  Light and sky intensities are drawn from
    U[1, 100]."""
    rng = scenes.SampleRng(0xD3A0_1000 + seed)
    kind = seed % 3
    s = RayScene()
    if kind == 0:
        ground = s.add_material(RayMaterial.lambertian((0.5, 0.5, 0.5)))
        s.add_sphere((0.0, -1000.0, 0.0), 1000.0, ground)
        lights = SamplingTargetList()
        for _ in range(int(rng.random_range(20.0, 120.0))):
            c = (rng.random_range(-8.0, 8.0), 0.0, rng.random_range(-8.0, 8.0))
            r = rng.random_range(0.15, 0.9)
            s.add_sphere((c[0], r, c[2]), r, s.add_material(_random_material(rng)))
        has_light = rng.random_double() < 0.5
        if has_light:
            e = rng.random_range(1.0, 100.0)
            c = (rng.random_range(-4.0, 4.0), rng.random_range(3.0, 6.0), rng.random_range(-4.0, 4.0))
            s.add_sphere(c, 0.5, s.add_material(RayMaterial.diffuse_light((e, e, e))))
            lights.add_sphere(c, 0.5)
        s.build_bvh()
        a = rng.random_range(0.0, 2.0 * math.pi)
        cam = (RayCamera(size, 1.0).with_max_depth(10).with_vertical_fov(rng.random_range(25.0, 50.0))
               .with_look_at((13.0 * math.cos(a), rng.random_range(1.0, 4.0), 13.0 * math.sin(a)), (0.0, 0.5, 0.0))
               .with_view_up((0.0, 1.0, 0.0)))
        if has_light:
            k = rng.random_range(0.1, 1.0)
            cam = cam.with_background((0.5 * k, 0.7 * k, 1.0 * k))
        return TrainingScene(s, cam, lights if has_light else None)
    if kind == 1:
        wall = lambda: RayMaterial.lambertian((rng.random_range(0.05, 0.8), rng.random_range(0.05, 0.8),
                                               rng.random_range(0.05, 0.8)))
        left, right, white = s.add_material(wall()), s.add_material(wall()), s.add_material(wall())
        e = rng.random_range(1.0, 100.0)
        light = s.add_material(RayMaterial.diffuse_light((e, e, e)))
        s.add_quad((555.0, 0.0, 0.0), (0.0, 555.0, 0.0), (0.0, 0.0, 555.0), left)
        s.add_quad((0.0, 0.0, 0.0), (0.0, 555.0, 0.0), (0.0, 0.0, 555.0), right)
        lw, ld = rng.random_range(60.0, 260.0), rng.random_range(60.0, 260.0)
        lq = ((278.0 + lw / 2, 554.0, 278.0 + ld / 2), (-lw, 0.0, 0.0), (0.0, 0.0, -ld))
        s.add_quad(*lq, light)
        s.add_quad((0.0, 0.0, 0.0), (555.0, 0.0, 0.0), (0.0, 0.0, 555.0), white)
        s.add_quad((555.0, 555.0, 555.0), (-555.0, 0.0, 0.0), (0.0, 0.0, -555.0), white)
        s.add_quad((0.0, 0.0, 555.0), (555.0, 0.0, 0.0), (0.0, 555.0, 0.0), white)
        for _ in range(int(rng.random_range(1.0, 5.0))):
            m = s.add_material(_random_material(rng))
            if rng.random_double() < 0.5:
                hgt = rng.random_range(80.0, 330.0)
                off = (rng.random_range(60.0, 400.0), 0.0, rng.random_range(60.0, 400.0))
                for corner, u, v in scenes.rotated_box_quads((0.0, 0.0, 0.0), (120.0, hgt, 120.0),
                                                             rng.random_range(-40.0, 40.0), off):
                    s.add_quad(corner, u, v, m)
            else:
                r = rng.random_range(40.0, 110.0)
                s.add_sphere((rng.random_range(r, 555.0 - r), r, rng.random_range(r, 555.0 - r)), r, m)
        s.build_bvh()
        lights = SamplingTargetList()
        lights.add_quad(*lq)
        cam = (RayCamera(size, 1.0).with_max_depth(50).with_background((0.0, 0.0, 0.0)).with_vertical_fov(40.0)
               .with_look_at((278.0 + rng.random_range(-120.0, 120.0), 278.0 + rng.random_range(-120.0, 120.0),
                              -800.0), (278.0, 278.0, 0.0))
               .with_view_up((0.0, 1.0, 0.0)))
        return TrainingScene(s, cam, lights)
    # kind 2: small mesh world under an HDR sky
    grad, perm = scenes.perlin_tables(seed)
    n = 48
    u = np.arange(n, dtype=np.float64) / float(n - 1) * rng.random_range(3.0, 8.0)
    U, V = np.meshgrid(u, u, indexing="xy")
    base = np.stack([U.ravel(), np.full(U.size, 0.5), V.ravel()], axis=-1)
    hts = np.zeros(U.size)
    for octave in range(4):
        hts = hts + 0.5 ** octave * scenes.perlin_noise(grad, perm, base * 2.0 ** octave)
    s.add_triangles_array(s.add_material(_random_material(rng)),
                          scenes.height_map_triangles(hts.reshape(n, n), 100.0, 100.0, 15.0))
    for _ in range(int(rng.random_range(2.0, 10.0))):
        c = (rng.random_range(-30.0, 30.0), rng.random_range(10.0, 24.0), rng.random_range(-30.0, 30.0))
        s.add_triangles_array(s.add_material(_random_material(rng)),
                              scenes.torus_triangles(c, rng.random_range(0.3, 1.5), rng.random_range(2.0, 6.0), 16, 32))
    s.build_bvh()
    env = EnvironmentLight(_sky(rng))
    a = rng.random_range(0.0, 2.0 * math.pi)
    cam = (RayCamera(size, 1.0).with_max_depth(8).with_vertical_fov(rng.random_range(30.0, 55.0))
           .with_look_at((70.0 * math.cos(a), rng.random_range(25.0, 45.0), 70.0 * math.sin(a)), (0.0, 10.0, 0.0))
           .with_view_up((0.0, 1.0, 0.0)))
    return TrainingScene(s, cam, None, env)


def render_pair(ts: TrainingScene, low_spp: int, high_spp: int, seed: int, context: Optional[Context] = None):
    """(beauty at low_spp, albedo, normal, target at high_spp) as float32 [h, w, 3] arrays.
    The target uses an independent RNG stream."""
    cam_lo = ts.camera.with_samples_per_pixel(low_spp).with_rng_seed(1 + 2 * seed)
    img, albedo, normal = PathTracer(cam_lo, context=context)._render(ts.scene, ts.lights, ts.environment, aovs=True)
    cam_hi = ts.camera.with_samples_per_pixel(high_spp).with_rng_seed(2 + 2 * seed)
    target = PathTracer(cam_hi, context=context)._render(ts.scene, ts.lights, ts.environment).pixels
    return img.pixels, albedo, normal, target


def render_split(ts: TrainingScene, spp: int, seed: int, context: Optional[Context] = None):
    """A render of `spp` samples per pixel with its split buffer and AOVs: (beauty,
    beauty_half, albedo, normal), beauty_half being the mean of the first spp // 2 samples
    of the same pixel streams (gt_render_accumulate twice on one accumulator)."""
    w, h, _ = ts.camera.image_size()
    cam = ts.camera.with_samples_per_pixel(spp).with_rng_seed(1 + 2 * seed)
    tracer = PathTracer(cam, context=context)
    acc = Accumulator(w, h, "f32", context=context)
    try:
        half = tracer.render_accumulate(ts.scene, acc, spp // 2, ts.lights, ts.environment).pixels.copy()
        full = tracer.render_accumulate(ts.scene, acc, spp - spp // 2, ts.lights, ts.environment).pixels
    finally:
        acc.close()
    _, albedo, normal = tracer._render(ts.scene, ts.lights, ts.environment, aovs=True)
    return full, half, albedo, normal


def evaluate(den: "Denoiser", ts: TrainingScene, spp: int, target: np.ndarray, seed: int, tile: int = 16,
             threshold: float = 3.0, context: Optional[Context] = None) -> dict:
    """relMSE against `target` of the plain render at `spp`, of its denoised image and of the
    denoised image with the per-tile fallback."""
    full, half, albedo, normal = render_split(ts, spp, seed, context)
    d, _ = den.denoise(full, albedo, normal)
    f, flags = den.denoise(full, albedo, normal, beauty_half=half, tile=tile, threshold=threshold)
    return {"plain": relmse(full, target), "denoised": relmse(d, target), "fallback": relmse(f, target),
            "fallback_tiles": int(flags.sum()), "tiles": int(flags.size)}


def render_training_set(count: int, size: int = 256, low_spp=(1, 2, 4, 8, 16, 32, 64, 128), high_spp: int = 1024,
                        first_seed: int = 0,
                        context: Optional[Context] = None, log=None):
    """`count` seeded scenes rendered by this path tracer; returns float32 arrays
    beauty, albedo, normal, target of shape [count, size, size, 3]."""
    out = [np.empty((count, size, size, 3), dtype=np.float32) for _ in range(4)]
    t0 = time.time()
    for i in range(count):
        seed = first_seed + i
        ts = training_scene(seed, size)
        parts = render_pair(ts, low_spp[seed % len(low_spp)], high_spp, seed, context)
        for k in range(4):
            out[k][i] = parts[k]
        if log and (i + 1) % 16 == 0:
            log(f"rendered {i + 1}/{count} training scenes in {time.time() - t0:.1f} s")
    return tuple(out)


def train(den: Denoiser, data, steps: int, batch: int = 16, crop: int = 128, lr: float = 2e-3, seed: int = 0,
          log=None, log_every: int = 100) -> list:
    """Adam on random crops (with flips) of the device training set `data` = (beauty,
    albedo, normal, target) CUDA tensors [count, h, w, 3]; the learning rate decays by
    cosine to lr / 20.  Returns the loss per step."""
    import torch

    beauty, albedo, normal, target = data
    count, h, w = beauty.shape[:3]
    g = torch.Generator(device="cpu").manual_seed(seed)
    losses = []
    for step in range(steps):
        idx = torch.randint(0, count, (batch,), generator=g)
        ys = torch.randint(0, h - crop + 1, (batch,), generator=g)
        xs = torch.randint(0, w - crop + 1, (batch,), generator=g)
        flips = torch.randint(0, 2, (batch, 2), generator=g)

        def crops(t):
            parts = []
            for b in range(batch):
                c = t[idx[b], ys[b]:ys[b] + crop, xs[b]:xs[b] + crop]
                if flips[b, 0]:
                    c = c.flip(0)
                if flips[b, 1]:
                    c = c.flip(1)
                parts.append(c)
            return torch.stack(parts).contiguous()

        b_, a_, n_, t_ = crops(beauty), crops(albedo), crops(normal), crops(target)
        # a flipped image's normals keep their world-space values: the network sees them
        # only as features, so the flip is a data augmentation, not a change of scene
        cur = lr * (0.05 + 0.95 * 0.5 * (1.0 + math.cos(math.pi * step / max(steps, 1))))
        losses.append(den.train_step(b_, t_, a_, n_, lr=cur))
        if log and (step + 1) % log_every == 0:
            log(f"step {step + 1}/{steps} loss {np.mean(losses[-log_every:]):.4f}")
    return losses


def relmse(x: np.ndarray, ref: np.ndarray) -> float:
    """mean((x - ref)^2 / (ref^2 + 0.01)) over pixels and channels."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.mean((x - ref) ** 2 / (ref * ref + 1e-2)))


def _accumulate(tracer, scene, acc, spp, lights, env, chunk):
    """Adds spp samples in chunks; returns (image, device ms)."""
    ms, img, done = 0.0, None, 0
    while done < spp:
        k = min(chunk, spp - done)
        img = tracer.render_accumulate(scene, acc, k, lights, env)
        ms += tracer.last_stats["gpu_ms"]
        done += k
    return img.pixels, ms


def convergence_sweep(den: Denoiser, scene, camera: RayCamera, lights=None, environment=None,
                      target_spp: int = 4096, max_spp: int = 1024, goal: float = 1e-3, tile: int = 16,
                      threshold: float = 3.0, trim: float = 1e-3, context: Optional[Context] = None,
                      log=None) -> dict:
    """Time to reach relMSE `goal`, plain accumulation against denoised.

    The reference image is two independent renders of target_spp / 2 samples, T1 and T2,
    averaged; its own error is estimated from their difference,
        e_T = mean((T1 - T2)^2 / 4 / (T^2 + 0.01)),
    and subtracted from every measured relMSE (relMSE(x, T) = err(x) + e_T for x independent
    of T).  The integrator's rare single-sample fireflies (caustics through glass onto the
    light, grazing GGX) dominate a plain mean of per-pixel errors, so the decision uses the
    mean over all but the `trim` fraction of pixels with the largest error; the untrimmed
    values are reported beside it.  Plain accumulation doubles its sample count from 1 to max_spp on one
    accumulator, so the image at N / 2 is the split buffer of the image at N.  The denoised
    time at N is the render time to N, a 1-sample AOV render and the denoise call (host
    buffers, copies included).  The camera must use random sampling."""
    import torch

    w, h, _ = camera.image_size()
    chunk = 256
    t_ref = []
    for k, seed in enumerate((0x7A11, 0x7A12)):
        acc = Accumulator(w, h, "f32", context=context)
        tr = PathTracer(camera.with_rng_seed(seed), context=context)
        img, ms = _accumulate(tr, scene, acc, target_spp // 2, lights, environment, chunk)
        acc.close()
        t_ref.append(img.astype(np.float64))
        if log:
            log(f"reference half {k + 1}: {target_spp // 2} spp in {ms / 1e3:.1f} s of device time")
    T = 0.5 * (t_ref[0] + t_ref[1])
    den_T = T * T + 1e-2
    ref_px = np.mean((t_ref[0] - t_ref[1]) ** 2 / 4.0 / den_T, axis=-1)  # the reference's own error
    e_T = float(np.mean(ref_px))

    def errs(x):
        """(trimmed, raw): relMSE against T less the reference's own error; trimmed drops the
        0.1% of pixels with the largest error (single-sample fireflies of the integrator)."""
        px = np.mean((np.asarray(x, dtype=np.float64) - T) ** 2 / den_T, axis=-1)
        keep = px <= np.quantile(px, 1.0 - trim)
        return float(np.mean(px[keep]) - np.mean(ref_px[keep])), float(np.mean(px)) - e_T

    tr = PathTracer(camera.with_rng_seed(0x5EED), context=context)
    t0 = time.perf_counter()
    _, albedo, normal = PathTracer(camera.with_samples_per_pixel(1).with_rng_seed(0x5EED), context=context)._render(
        scene, lights, environment, aovs=True)
    aov_s = time.perf_counter() - t0
    den.denoise(np.zeros((h, w, 3), np.float32))  # sizes the denoiser's buffers outside the timings
    acc = Accumulator(w, h, "f32", context=context)
    rows, prev, n, render_ms = [], None, 1, 0.0
    try:
        while n <= max_spp:
            img, ms = _accumulate(tr, scene, acc, n - acc.samples, lights, environment, chunk)
            render_ms += ms
            pe, pr = errs(img)
            row = {"spp": n, "render_s": render_ms / 1e3, "plain": pe, "plain_raw": pr}
            if prev is not None:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                d, flags = den.denoise(img, albedo, normal, beauty_half=prev, tile=tile, threshold=threshold)
                dn_s = time.perf_counter() - t0
                de, dr = errs(d)
                row.update(denoised=de, denoised_raw=dr, denoise_s=dn_s, fallback_tiles=int(flags.sum()),
                           denoised_time_s=render_ms / 1e3 + aov_s + dn_s)
            rows.append(row)
            if log:
                log(" ".join(f"{k} {v:.4g}" if isinstance(v, float) else f"{k} {v}" for k, v in row.items()))
            prev = img.copy()
            n *= 2
    finally:
        acc.close()
    # relMSE ~ C / N for plain accumulation: C from the last three points of the sweep
    c_fit = float(np.median([r["plain"] * r["spp"] for r in rows[-3:]]))
    s_per_spp = rows[-1]["render_s"] / rows[-1]["spp"]

    def plain_time(g):
        hit = next((r for r in rows if r["plain"] <= g), None)
        if hit is not None:
            return {"time_s": hit["render_s"], "spp": hit["spp"], "extrapolated": False}
        if c_fit <= 0.0:
            return None
        n_star = c_fit / g
        return {"time_s": s_per_spp * n_star, "spp": n_star, "extrapolated": True}

    def denoised_time(g):
        hit = next((r for r in rows if "denoised" in r and r["denoised"] <= g), None)
        return {"time_s": hit["denoised_time_s"], "spp": hit["spp"]} if hit is not None else None

    goals = {}
    for g in sorted({goal, 1e-2, 5e-3, 2e-3, 1e-3}, reverse=True):
        pt, dt = plain_time(g), denoised_time(g)
        goals[f"{g:g}"] = {"plain": pt, "denoised": dt,
                           "speedup": (pt["time_s"] / dt["time_s"]) if pt and dt else None}
    return {"goal": goal, "trim": trim, "reference_error": e_T, "aov_s": aov_s, "curve": rows,
            "plain_c": c_fit, "plain": plain_time(goal), "denoised": denoised_time(goal),
            "speedup": goals[f"{goal:g}"]["speedup"], "goals": goals,
            "best_denoised": min((r["denoised"] for r in rows if "denoised" in r), default=None)}


def main(argv=None) -> int:
    import argparse

    import torch

    ap = argparse.ArgumentParser(description="Train the denoiser on scenes rendered by this path tracer.")
    ap.add_argument("--scenes", type=int, default=1536)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--high-spp", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=24000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--crop", type=int, default=128)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", type=str, default=str(DEFAULT_WEIGHTS))
    args = ap.parse_args(argv)
    log = lambda m: print(m, flush=True)
    t0 = time.time()
    data = render_training_set(args.scenes, args.size, high_spp=args.high_spp, log=log)
    log(f"training set: {args.scenes} scenes in {time.time() - t0:.1f} s")
    dev = [torch.from_numpy(a).cuda() for a in data]
    den = Denoiser(args.seed)
    t1 = time.time()
    losses = train(den, dev, args.steps, args.batch, args.crop, args.lr, args.seed, log)
    torch.cuda.synchronize()
    log(f"trained {args.steps} steps in {time.time() - t1:.1f} s; final loss {np.mean(losses[-100:]):.4f}")
    Path(args.out).parent.mkdir(parents=True, exist_ok=True)
    den.save(args.out)
    log(f"saved {args.out}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
