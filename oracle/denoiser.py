"""FP64 numpy restatement of the learned shadow + AO denoiser (test infrastructure).

Same network, feature gather (3x3 taps, clamped to the image, channel 5 replaced by
the depth relative to the centre pixel, zero rows for background pixels), softmax
7x7 filter (the AO average and the ratio estimator sum(w S) / sum(w U) of the
shadowed over the unshadowed direct light) and weighted squared-error loss as
luz_gb300/csrc/denoise.cu, evaluated in
double precision with exact backpropagation. Inputs are the device's BF16 feature
planes and weights rounded to BF16, as the device uses them; the device also rounds
activations to BF16 between layers, so agreement is to BF16 accuracy.
"""
from __future__ import annotations

import numpy as np

SHAPES = [(64, 72), (64, 64), (64, 64), (49, 64)]


def bf16_round(x: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def bf16_bits_to_f32(b: np.ndarray) -> np.ndarray:
    return (np.ascontiguousarray(b).view(np.uint16).astype(np.uint32) << 16).view(np.float32)


def unpack(params: np.ndarray):
    out, o = [], 0
    for n, k in SHAPES:
        W = params[o:o + n * k].reshape(n, k)
        o += n * k
        b = params[o:o + n]
        o += n
        out.append((W, b))
    return out


def gather(feat_bits: np.ndarray, lin_depth: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """feat_bits [N,H,W,8] bf16 bits, lin_depth [N,H,W] → X [N,H,W,72] (BF16 values), valid mask."""
    f = bf16_bits_to_f32(feat_bits).astype(np.float32)
    N, H, W, _ = f.shape
    valid = lin_depth > 0
    X = np.zeros((N, H, W, 72), np.float32)
    ys, xs = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        qy = np.clip(ys + dy, 0, H - 1)
        qx = np.clip(xs + dx, 0, W - 1)
        v = f[:, qy, qx, :].copy()
        dq = lin_depth[:, qy, qx]
        dc = lin_depth
        with np.errstate(divide="ignore", invalid="ignore"):
            rel = np.where(dq > 0, np.clip((dq - dc) / np.where(dc > 0, dc, 1), -1, 1), 0).astype(np.float32)
        v[..., 5] = bf16_round(rel)
        X[..., tap * 8:(tap + 1) * 8] = v
    X[~valid] = 0
    return X, valid


# Loss weight of each shadow-ratio output (the AO output has weight 1).
SHADOW_WEIGHT = 1.0 / 3.0


def neighbours(sig: np.ndarray) -> np.ndarray:
    """[N,H,W,4] → [N,H,W,49,4] at the 7x7 taps (clamped)."""
    N, H, W, C4 = sig.shape
    ys, xs = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    out = np.zeros((N, H, W, 49, C4), np.float64)
    for k in range(49):
        qy = np.clip(ys + k // 7 - 3, 0, H - 1)
        qx = np.clip(xs + k % 7 - 3, 0, W - 1)
        out[..., k, :] = sig[:, qy, qx, :]
    return out


def forward_backward(params: np.ndarray, feat_bits, lin_depth, noisy, unshadowed, target, weight=None,
                     shadow_weight: float = SHADOW_WEIGHT):
    """noisy: [N,H,W,4] shadowed direct light S (r, g, b) and AO; unshadowed: [N,H,W,4]
    unshadowed direct light U (r, g, b, -); target: [N,H,W,4] shadow ratio (r, g, b) and
    AO. Outputs per pixel: the ratio estimator R_c = sum(w S_c) / sum(w U_c) (1 where
    the sum is 0) and AO' = sum(w AO). Returns (y [N,H,W,4], loss, grad [16177]);
    loss = sum over valid pixels and outputs of weight x (y - t)^2 divided by the
    number of pixels (background pixels count as zero error); weight [N,H,W,4] per
    pixel, or shadow_weight for the ratio outputs and 1 for AO."""
    layers = [(bf16_round(W).astype(np.float64), b.astype(np.float64)) for W, b in unpack(params)]
    X, valid = gather(feat_bits, lin_depth)
    x = X[valid].astype(np.float64)                       # [P, 72]
    A = neighbours(noisy)[valid]                          # [P, 49, 4]
    Uk = neighbours(unshadowed)[valid][..., :3]           # [P, 49, 3]
    t = target[valid].astype(np.float64)                  # [P, 4]
    cw = (np.asarray(weight, np.float64)[valid] if weight is not None else
          np.array([shadow_weight, shadow_weight, shadow_weight, 1.0]))
    hs = [x]
    h = x
    for W, b in layers[:3]:
        h = np.maximum(h @ W.T + b, 0.0)
        hs.append(h)
    W4, b4 = layers[3]
    z = h @ W4.T + b4
    z -= z.max(axis=1, keepdims=True)
    e = np.exp(z)
    w = e / e.sum(axis=1, keepdims=True)
    sums = (w[:, :, None] * A).sum(axis=1)                # [P, 4]: sum(w S), sum(w AO)
    du = (w[:, :, None] * Uk).sum(axis=1)                 # [P, 3]: sum(w U)
    lit = du > 0
    ratio = np.where(lit, np.clip(sums[:, :3] / np.where(lit, du, 1.0), 0.0, 1.0), 1.0)
    y = np.concatenate([ratio, sums[:, 3:4]], axis=1)     # [P, 4]
    npx = noisy.shape[0] * noisy.shape[1] * noisy.shape[2]   # every pixel of the batch, as the device's mean
    err = y - t
    loss = float((cw * err ** 2).sum()) / npx
    dy = 2.0 * cw * err / npx
    dq = np.where(lit, dy[:, :3] / np.where(lit, du, 1.0), 0.0)      # d loss / d sum(w S)
    dw = dy[:, None, 3] * A[..., 3] + (dq[:, None, :] * (A[..., :3] - ratio[:, None, :] * Uk)).sum(axis=2)
    dz = w * (dw - (w * dw).sum(axis=1, keepdims=True))
    grads = []
    d = dz
    for li in range(3, -1, -1):
        W, b = layers[li]
        hin = hs[li]
        grads.append((d.T @ hin, d.sum(axis=0)))
        if li > 0:
            d = (d @ W) * (hs[li] > 0)
    grads.reverse()
    g = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    yfull = np.zeros(noisy.shape)
    yfull[valid] = y
    return yfull, loss, g
