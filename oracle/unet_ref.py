"""CPU oracle of the U-Net psi guess (test infrastructure only: the tests compare the GPU network
against it; nothing in the library calls it).

The same network as include/ptgpu_unet.h, written with numpy in FP64 with BF16 rounding at the
points where the GPU rounds: the gathered convolution inputs (including the 2x2 average, summed
((a+b)+c)+d in FP32 and scaled by 1/4), the weights, the post-ReLU activations, and the masked
output gradients that enter the backward GEMMs.  Accumulations are FP64 here and FP32 on the
GPU, so the two agree to rounding (occasional one-ulp BF16 flips of an activation).

Layout: activations (B, H, W, C); parameters flat as in ptgpu_unet.h.
"""

from __future__ import annotations

import numpy as np

# (src0, src1, mode, cin, cout, level, out); mode 0 plain, 1 2x2 average pool, 2 upsample+concat
SPEC = [(-1, -1, 0, 4, 32, 0, 0), (0, -1, 0, 32, 32, 0, 1), (1, -1, 1, 32, 64, 1, 2), (2, -1, 0, 64, 64, 1, 3),
        (3, -1, 1, 64, 128, 2, 4), (4, -1, 0, 128, 128, 2, 5), (5, -1, 1, 128, 256, 3, 6), (6, -1, 0, 256, 256, 3, 7),
        (7, 5, 2, 384, 128, 2, 8), (8, -1, 0, 128, 128, 2, 9), (9, 3, 2, 192, 64, 1, 10), (10, -1, 0, 64, 64, 1, 11),
        (11, 1, 2, 96, 32, 0, 12), (12, -1, 0, 32, 32, 0, 13)]

EXACT = False  # True: no BF16 rounding anywhere (an FP64 network, for finite-difference checks)


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as FP64 values."""
    if EXACT:
        return np.asarray(x, dtype=np.float64)
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layout():
    """Offsets of each convolution's (weights, bias), the output layer's w and b, the total."""
    off, offs = 0, []
    for (_, _, _, cin, cout, _, _) in SPEC:
        wo = off
        off += cout * 9 * cin
        offs.append((wo, off))
        off += cout
    return offs, off, off + 32, off + 33


def _view(acts, x0, s0, s1, mode):
    a0 = x0 if s0 < 0 else acts[s0]
    if mode == 0:
        return a0
    if mode == 1:  # average of 2x2 in FP32 ((a+b)+c)+d, then x 0.25, rounded to BF16 by the gather
        f = a0 if EXACT else a0.astype(np.float32)
        s = ((f[:, 0::2, 0::2] + f[:, 0::2, 1::2]) + f[:, 1::2, 0::2]) + f[:, 1::2, 1::2]
        return bf16(s * 0.25)
    up = np.repeat(np.repeat(a0, 2, axis=1), 2, axis=2)
    return np.concatenate([up, acts[s1]], axis=3)


def _im2col(v):
    """(B,H,W,C) -> (B*H*W, 9*C), column = tap*C + c, tap = 3*(dy+1)+(dx+1), zero padding."""
    B, H, W, C = v.shape
    p = np.zeros((B, H + 2, W + 2, C))
    p[:, 1:-1, 1:-1] = v
    cols = [p[:, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W] for dy in (-1, 0, 1) for dx in (-1, 0, 1)]
    return np.concatenate(cols, axis=3).reshape(B * H * W, 9 * C)


def forward(params: np.ndarray, x: np.ndarray):
    """x (B,4,H,W) FP32 -> (y (B,H,W), cache)."""
    offs, out_w, out_b, _ = layout()
    x0 = bf16(np.transpose(x, (0, 2, 3, 1)))
    acts = [None] * 14
    views = []
    for li, (s0, s1, mode, cin, cout, lev, out) in enumerate(SPEC):
        v = _view(acts, x0, s0, s1, mode)
        B, H, W, _ = v.shape
        wo, bo = offs[li]
        w = bf16(params[wo:wo + cout * 9 * cin]).reshape(cout, 9 * cin)
        z = _im2col(v) @ w.T + params[bo:bo + cout].astype(np.float64)
        acts[out] = bf16(np.maximum(z, 0.0)).reshape(B, H, W, cout)
        views.append(v)
    y = acts[13] @ params[out_w:out_w + 32].astype(np.float64) + float(params[out_b])
    return y, (x0, acts, views)


def gradients(params: np.ndarray, x: np.ndarray, target: np.ndarray):
    """(loss, flat gradient) of mean (y - target)^2."""
    offs, out_w, out_b, total = layout()
    y, (x0, acts, views) = forward(params, x)
    d = y - target.astype(np.float64)
    loss = float(np.mean(d * d))
    dy = 2.0 * d / y.size
    g = np.zeros(total)
    g[out_w:out_w + 32] = np.einsum("bhw,bhwc->c", dy, acts[13])
    g[out_b] = dy.sum()
    grads = [np.zeros_like(a) for a in acts]
    grads[13] = dy[..., None] * params[out_w:out_w + 32].astype(np.float64)
    for li in range(len(SPEC) - 1, -1, -1):
        s0, s1, mode, cin, cout, lev, out = SPEC[li]
        v = views[li]
        B, H, W, _ = v.shape
        wo, bo = offs[li]
        dz_exact = np.where(acts[out] > 0, grads[out], 0.0).reshape(-1, cout)
        dz = bf16(dz_exact)
        g[wo:wo + cout * 9 * cin] = (dz.T @ _im2col(v)).reshape(-1)
        g[bo:bo + cout] = dz_exact.sum(axis=0)
        if s0 < 0:
            continue
        w = bf16(params[wo:wo + cout * 9 * cin]).reshape(cout, 9, cin)
        dzp = np.zeros((B, H + 2, W + 2, cout))
        dzp[:, 1:-1, 1:-1] = dz.reshape(B, H, W, cout)
        dX = np.zeros((B, H, W, cin))
        for t in range(9):  # dX[q] += dZ[q - off(t)] W[:, t, :]
            dyy, dxx = t // 3 - 1, t % 3 - 1
            dX += dzp[:, 1 - dyy:1 - dyy + H, 1 - dxx:1 - dxx + W] @ w[:, t, :]
        if mode == 0:
            grads[s0] += dX
        elif mode == 1:
            grads[s0] += 0.25 * np.repeat(np.repeat(dX, 2, axis=1), 2, axis=2)
        else:
            c0 = acts[s0].shape[3]
            up = dX[..., :c0]
            grads[s0] += ((up[:, 0::2, 0::2] + up[:, 0::2, 1::2]) + up[:, 1::2, 0::2]) + up[:, 1::2, 1::2]
            grads[s1] += dX[..., c0:]
    return loss, g
