"""CPU reference of the learned update network (numpy).

TEST INFRASTRUCTURE ONLY: used by tests/ to check libtomo.so's network
kernels; the product never imports it.  The network has no counterpart in
the reference project; this file states its mathematics directly.

Network: 5 layers of 3x3 convolutions with zero padding, NHWC activations.
  x0 = features (3 channels, zero-padded to 16)
  y_l = relu(conv(y_{l-1}, W_l) + b_l)   l = 1..4, 32 channels
  out = conv(y_4, W5) + b5              1 channel
Loss: masked mean squared error  sum(mask * (out - t)^2) / sum(mask).

With emulate=True the BF16 rounding points of the GPU kernels are applied
(features, weights of layers 1-4, activations, and the propagated gradients
dz_l); sums are taken in FP64.  With emulate=False everything is FP64.
"""
from __future__ import annotations

import numpy as np

C = 32
SHAPES = [("W1", (9, 16, C)), ("b1", (C,)), ("W2", (9, C, C)), ("b2", (C,)), ("W3", (9, C, C)), ("b3", (C,)),
          ("W4", (9, C, C)), ("b4", (C,)), ("W5", (9, C)), ("b5", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16(x):
    """Round to bfloat16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + n], np.float64).reshape(shp)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SHAPES])


def _shift(x, dy, dx):
    """x[b, y+dy, x+dx, :] with zeros outside (NHWC)."""
    B, H, W, Cc = x.shape
    out = np.zeros_like(x)
    ys, yd = (slice(dy, H), slice(0, H - dy)) if dy >= 0 else (slice(0, H + dy), slice(-dy, H))
    xs, xd = (slice(dx, W), slice(0, W - dx)) if dx >= 0 else (slice(0, W + dx), slice(-dx, W))
    out[:, yd, xd, :] = x[:, ys, xs, :]
    return out


def conv(x, w):
    """out[p, co] = sum_tap sum_ci x[p + off(tap), ci] w[tap, ci, co]; off = (tap//3 - 1, tap%3 - 1)."""
    out = 0.0
    for tap in range(9):
        out = out + np.tensordot(_shift(x, tap // 3 - 1, tap % 3 - 1), w[tap], axes=([3], [0]))
    return out


def conv_t(d, w):
    """Adjoint of conv w.r.t. x: dx[p, ci] = sum_tap sum_co d[p - off(tap), co] w[tap, ci, co]."""
    out = 0.0
    for tap in range(9):
        out = out + np.tensordot(_shift(d, -(tap // 3 - 1), -(tap % 3 - 1)), w[tap], axes=([3], [1]))
    return out


def wgrad(x, d):
    """dW[tap, ci, co] = sum_p x[p + off(tap), ci] d[p, co]."""
    return np.stack([np.tensordot(_shift(x, tap // 3 - 1, tap % 3 - 1), d, axes=([0, 1, 2], [0, 1, 2]))
                     for tap in range(9)])


def features_nhwc(feat):
    """Planar [B][3][H][W] -> NHWC with 16 channels."""
    B, _, H, W = feat.shape
    x = np.zeros((B, H, W, 16))
    x[..., :3] = np.transpose(feat, (0, 2, 3, 1))
    return x


def forward(p, feat, emulate=True):
    P = unpack(p)
    r = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
    x = r(features_nhwc(np.asarray(feat, np.float64)))
    ys = [x]
    for l in range(1, 5):
        z = conv(ys[-1], r(P[f"W{l}"])) + P[f"b{l}"]
        ys.append(r(np.maximum(z, 0.0)))
    out = conv(ys[4], P["W5"][:, :, None])[..., 0] + P["b5"][0]
    return out, ys


def loss_and_grad(p, feat, tgt, mask, emulate=True):
    P = unpack(p)
    r = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
    out, ys = forward(p, feat, emulate)
    msum = float(np.sum(mask))
    e = (out - tgt) * mask
    loss = float(np.sum(e * e)) / msum
    dout = 2.0 * e / msum
    g = {}
    g["W5"] = wgrad(ys[4], dout[..., None])[:, :, 0]
    g["b5"] = np.array([dout.sum()])
    dz = r((ys[4] > 0) * conv_t(dout[..., None], P["W5"][:, :, None]))
    for l in range(4, 0, -1):
        g[f"W{l}"] = wgrad(ys[l - 1], dz)
        g[f"b{l}"] = dz.sum(axis=(0, 1, 2))
        if l > 1:
            dz = r((ys[l - 1] > 0) * conv_t(dz, r(P[f"W{l}"])))
    return loss, pack(g)
