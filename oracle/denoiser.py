"""TEST INFRASTRUCTURE ONLY — the CPU oracle of the learned denoiser.

The reference has no denoiser (it stops at the AOVs of PathTracer::render_denoising_aovs,
raytracing/renderer.rs:121-129), so this oracle restates the library's own network
definition in float64 with torch's CPU autograd, parameter for parameter in the flat
layout gt_denoiser_get_params returns, and the split-buffer per-tile fallback test in
numpy.  Only tests/ may use it, as the checker of the GPU kernels.

Definitions restated here:
  input     x = [log1p(max(beauty, 0)), albedo, normal]  (9 channels; non-finite beauty = 0;
            images padded to multiples of 16 by repeating the last row and column)
  network   5 levels of two 3x3 convs + ReLU (32/48/64/80/96 channels), 2x2 average
            pooling between levels, nearest 2x upsampling concatenated (upsampled first,
            then the skip) before the two decoder convs of each level, a final 3x3 conv
            to 3 channels without ReLU
  output    out = conv_out + log1p(max(beauty, 0));  image = max(expm1(out), 0)
  loss      mean |out - log1p(max(target, 0))| over pixels and channels

BF16-faithful mode (bf16=True): the same network with values and gradients rounded to
BF16 where the library stores BF16 tensors — the network input, the weights (their
gradient reaches the FP32 masters unrounded), every ReLU'd convolution output, the
pooled tensors, and in the backward pass the gradient of each stored activation, of the
concatenated decoder inputs, of the pooled tensors and of the prediction (the loss
gradient).  Convolutions accumulate in float64 (the library in FP32), bias and residual
stay unrounded.
"""
from __future__ import annotations

import numpy as np

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


def _unflatten(params):
    """Flat [cout][3][3][cin] + [cout] per layer -> torch conv weights [cout][cin][3][3]."""
    out, off = [], 0
    for cin, cout, relu in layer_shapes():
        n = cout * 9 * cin
        w = params[off:off + n].reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
        off += n
        b = params[off:off + cout]
        off += cout
        out.append((w, b, relu))
    assert off == params.numel()
    return out


def _pad16(t):
    """[n, c, h, w] -> padded to multiples of 16 by repeating the last row / column."""
    import torch

    h, w = t.shape[2], t.shape[3]
    hp, wp = (h + 15) // 16 * 16, (w + 15) // 16 * 16
    if hp != h:
        t = torch.cat([t, t[:, :, -1:, :].expand(-1, -1, hp - h, -1)], dim=2)
    if wp != w:
        t = torch.cat([t, t[:, :, :, -1:].expand(-1, -1, -1, wp - w)], dim=3)
    return t


def _log1p_clean(x):
    import torch

    x = torch.where(torch.isfinite(x), x, torch.zeros_like(x))
    return torch.log1p(torch.clamp(x, min=0.0))


def _bf16(t):
    import torch

    return t.to(torch.bfloat16).to(torch.float64)


def _rounders():
    """(value and gradient, value only, gradient only) BF16 rounding as autograd functions."""
    import torch

    class Both(torch.autograd.Function):
        @staticmethod
        def forward(ctx, t):
            return _bf16(t)

        @staticmethod
        def backward(ctx, g):
            return _bf16(g)

    class Value(torch.autograd.Function):
        @staticmethod
        def forward(ctx, t):
            return _bf16(t)

        @staticmethod
        def backward(ctx, g):
            return g

    class Grad(torch.autograd.Function):
        @staticmethod
        def forward(ctx, t):
            return t.clone()

        @staticmethod
        def backward(ctx, g):
            return _bf16(g)

    return Both.apply, Value.apply, Grad.apply


def forward_log(params, beauty, albedo=None, normal=None, bf16=False):
    """Log-space output [n, hp, wp, 3] (float64 torch) for inputs [n, h, w, 3]; bf16 rounds
    where the library stores BF16 (the module docstring lists the points)."""
    import torch
    import torch.nn.functional as F

    if bf16:
        both, value, grad = _rounders()
    else:
        both = value = grad = lambda t: t

    b = torch.as_tensor(beauty, dtype=torch.float64)
    z = torch.zeros_like(b)
    a = torch.as_tensor(albedo, dtype=torch.float64) if albedo is not None else z
    nm = torch.as_tensor(normal, dtype=torch.float64) if normal is not None else z
    lb = _log1p_clean(b)
    x = torch.cat([lb, a, nm], dim=-1).permute(0, 3, 1, 2)
    x = _pad16(x)
    lbp = x[:, :3]
    x = value(x)
    layers = _unflatten(params)

    def conv(i, t):
        w, bias, relu = layers[i]
        y = F.conv2d(t, value(w), bias, padding=1)
        return both(F.relu(y)) if relu else y

    L = len(CHANNELS)
    skips = []
    t = x
    for lv in range(L):
        if lv > 0:
            t = both(F.avg_pool2d(t, 2))
        t = conv(2 * lv + 1, conv(2 * lv, t))
        skips.append(t)
    for k, lv in enumerate(range(L - 2, -1, -1)):
        up = F.interpolate(t, scale_factor=2, mode="nearest")
        t = grad(torch.cat([up, skips[lv]], dim=1))
        base = 2 * L + 2 * k
        t = conv(base + 1, conv(base, t))
    out = grad(conv(len(layers) - 1, t) + lbp)
    return out.permute(0, 2, 3, 1)


def denoise(params, beauty, albedo=None, normal=None, bf16=False) -> np.ndarray:
    """The denoised image [h, w, 3] of one frame (float64 numpy); bf16 as in forward_log."""
    import torch

    p = torch.as_tensor(np.asarray(params, dtype=np.float64))
    add = lambda t: None if t is None else np.asarray(t, dtype=np.float64)[None]
    h, w = beauty.shape[:2]
    with torch.no_grad():
        out = forward_log(p, add(beauty), add(albedo), add(normal), bf16=bf16)[0, :h, :w]
    return np.maximum(np.expm1(out.numpy()), 0.0)


def loss_and_grad(params, beauty, target, albedo=None, normal=None, bf16=False):
    """(loss, flat gradient) in float64 for a batch [n, h, w, 3] (h, w multiples of 16);
    bf16 as in forward_log."""
    import torch

    p = torch.tensor(np.asarray(params, dtype=np.float64), requires_grad=True)
    out = forward_log(p, beauty, albedo, normal, bf16=bf16)
    tgt = _log1p_clean(torch.as_tensor(target, dtype=torch.float64))
    loss = (out - tgt).abs().mean()
    loss.backward()
    return float(loss.detach()), p.grad.numpy().copy()


def _tile_stats(denoised, plain, half, tile, threshold):
    d = np.asarray(denoised, dtype=np.float64)
    p = np.asarray(plain, dtype=np.float64)
    a = np.asarray(half, dtype=np.float64)
    p = np.where(np.isfinite(p), p, 0.0)
    a = np.where(np.isfinite(a), a, 0.0)
    h, w = p.shape[:2]
    ty, tx = (h + tile - 1) // tile, (w + tile - 1) // tile
    shift = np.zeros((ty, tx))
    bound = np.zeros((ty, tx))
    for j in range(ty):
        for i in range(tx):
            sl = (slice(j * tile, (j + 1) * tile), slice(i * tile, (i + 1) * tile))
            n = p[sl].shape[0] * p[sl].shape[1]
            md = d[sl].reshape(-1, 3).mean(axis=0)
            mp = p[sl].reshape(-1, 3).mean(axis=0)
            v = ((a[sl] - p[sl]) ** 2).reshape(-1, 3).sum(axis=0) / (n * n)
            shift[j, i] = np.sum((md - mp) ** 2)
            bound[j, i] = threshold * threshold * np.sum(v + (0.01 * mp) ** 2)
    return d, p, shift, bound


def tile_fallback(denoised, plain, half, tile: int = 16, threshold: float = 3.0):
    """The split-buffer residual test per tile: (image, flags).  Per channel the tile means
    m_d (denoised) and m_p (plain) and v = sum((a - p)^2) / N^2, the variance of m_p
    estimated from the two halves; the tile keeps the plain render when
    sum_c (m_d - m_p)^2 > threshold^2 * sum_c (v + (0.01 m_p)^2)."""
    d, p, shift, bound = _tile_stats(denoised, plain, half, tile, threshold)
    flags = (shift > bound).astype(np.uint8)
    out = d.copy()
    for j, i in zip(*np.nonzero(flags)):
        sl = (slice(j * tile, (j + 1) * tile), slice(i * tile, (i + 1) * tile))
        out[sl] = p[sl]
    return out, flags


def tile_margin(denoised, plain, half, tile: int = 16, threshold: float = 3.0) -> np.ndarray:
    """Per tile |shift - bound| / (shift + bound): how far each tile's decision is from the
    boundary (small values may round either way in FP32)."""
    _, _, shift, bound = _tile_stats(denoised, plain, half, tile, threshold)
    return np.abs(shift - bound) / np.maximum(shift + bound, 1e-300)
