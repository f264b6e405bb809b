"""CPU restatement of the learned reconstruction net (forward, loss, backward,
Adam) -- TEST INFRASTRUCTURE ONLY.

The reference renderer has no learned part; this file is the checker for the
project's own CUDA kernels (csrc/svo_net.cuh): the tests compare the GPU
gradients, outputs and optimiser steps with it on the same inputs. Nothing in
the product imports it.

Net: four 3x3 "same" convolutions with zero padding at the frame border,
channels 8 -> 16 -> 16 -> 16 -> 4, ReLU after the first three. Inputs
(8 planes): R, G, B, depth, hole mask, motion magnitude, sub-pixel offset, ray
elevation. Outputs
(4 planes): R, G, B (the input colour plus the last layer's first three
channels) and a confidence logit.

Numerics shared with the GPU: weights, input features and hidden activations
are rounded to bfloat16 (round to nearest even) before they are used; sums are
exact here (float64) and FP32 on the GPU. Gradients pass the roundings
unchanged (straight-through).

Flat parameter layout (float32, NET_PARAMS values): for each layer l,
W_l as [9 taps][C_in][C_out] (tap = (dy+1)*3 + (dx+1)), then b_l[C_out].
"""
from __future__ import annotations

import numpy as np

CHANNELS = (8, 16, 16, 16, 4)
LAYERS = 4


def layer_shapes():
    return [((9, CHANNELS[l], CHANNELS[l + 1]), (CHANNELS[l + 1],)) for l in range(LAYERS)]


NET_PARAMS = sum(9 * CHANNELS[l] * CHANNELS[l + 1] + CHANNELS[l + 1] for l in range(LAYERS))


def unpack(params: np.ndarray):
    """Flat vector -> [(W [9,Cin,Cout], b [Cout]), ...] (views)."""
    out, o = [], 0
    for ws, bs in layer_shapes():
        nw = int(np.prod(ws))
        out.append((params[o:o + nw].reshape(ws), params[o + nw:o + nw + bs[0]]))
        o += nw + bs[0]
    return out


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest even) and back, via float32 bits."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _shift(a: np.ndarray, dy: int, dx: int) -> np.ndarray:
    """out[..., y, x] = a[..., y+dy, x+dx], zero outside the frame."""
    H, W = a.shape[-2:]
    out = np.zeros_like(a)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    if ys < ye and xs < xe:
        out[..., ys:ye, xs:xe] = a[..., ys + dy:ye + dy, xs + dx:xe + dx]
    return out


TAPS = [(t // 3 - 1, t % 3 - 1) for t in range(9)]


def conv(a: np.ndarray, w: np.ndarray, b: np.ndarray) -> np.ndarray:
    """a [Cin,H,W], w [9,Cin,Cout], b [Cout] -> [Cout,H,W]."""
    out = np.zeros((w.shape[2],) + a.shape[1:], np.float64)
    for t, (dy, dx) in enumerate(TAPS):
        out += np.einsum("chw,co->ohw", _shift(a, dy, dx), w[t])
    return out + b[:, None, None]


def forward(params: np.ndarray, feat: np.ndarray, rounding: bool = True):
    """feat [8,H,W] -> (out [4,H,W], cache for backward)."""
    rnd = bf16 if rounding else (lambda v: np.asarray(v, np.float64))
    layers = unpack(np.asarray(params, np.float32))
    x = rnd(feat)
    acts = [x]
    a = x
    for l, (w, b) in enumerate(layers):
        pre = conv(a, rnd(w), np.asarray(b, np.float64))
        if l < LAYERS - 1:
            a = rnd(np.maximum(pre, 0.0))
            acts.append(a)
        else:
            out = pre.copy()
            out[:3] += x[:3]
    return out, acts


def target_rgb(bgrx: np.ndarray, H: int, W: int) -> np.ndarray:
    """BGRX8 words -> [3,H,W] R,G,B in [0,1]."""
    w = np.asarray(bgrx, np.uint32).reshape(H, W)
    return np.stack([(w >> 16) & 255, (w >> 8) & 255, w & 255]).astype(np.float64) / 255.0


def loss_grad(out: np.ndarray, tgt: np.ndarray, tau: float, lam: float):
    """Mean over pixels of sum_c (rgb_c - t_c)^2 / 3 + lam * BCE(logit, label),
    label = max_c |rgb_c - t_c| < tau. Returns (loss_rgb, loss_conf, d_out)."""
    n = out.shape[1] * out.shape[2]
    diff = out[:3] - tgt
    label = (np.abs(diff).max(0) < tau).astype(np.float64)
    z = out[3]
    l_rgb = float((diff ** 2).sum() / 3.0 / n)
    l_conf = float((np.logaddexp(0.0, z) - label * z).sum() / n)
    d = np.zeros_like(out)
    d[:3] = 2.0 / 3.0 * diff / n
    d[3] = lam * (1.0 / (1.0 + np.exp(-z)) - label) / n
    return l_rgb, l_conf, d


def backward(params: np.ndarray, acts, d_out: np.ndarray, rounding: bool = True) -> np.ndarray:
    """Gradient of the loss w.r.t. the flat parameter vector."""
    rnd = bf16 if rounding else (lambda v: np.asarray(v, np.float64))
    layers = unpack(np.asarray(params, np.float32))
    grads = []
    g = d_out
    for l in range(LAYERS - 1, -1, -1):
        w, _ = layers[l]
        a_in = acts[l]
        if l < LAYERS - 1:
            g = g * (acts[l + 1] > 0)
        gw = np.zeros(w.shape, np.float64)
        for t, (dy, dx) in enumerate(TAPS):
            gw[t] = np.einsum("chw,ohw->co", _shift(a_in, dy, dx), g)
        gb = g.sum(axis=(1, 2))
        grads.append((gw, gb))
        if l > 0:
            wr = rnd(w)
            ga = np.zeros_like(a_in)
            for t, (dy, dx) in enumerate(TAPS):
                ga += _shift(np.einsum("ohw,co->chw", g, wr[t]), -dy, -dx)
            g = ga
    flat = []
    for gw, gb in reversed(grads):
        flat.append(gw.reshape(-1))
        flat.append(gb)
    return np.concatenate(flat)


def adam(params, m, v, g, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step (step counts from 1); returns new (params, m, v)."""
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v


def init_params(seed: int) -> np.ndarray:
    """He-normal weights, zero biases, last layer scaled down (starts near
    the identity on colour and a neutral confidence)."""
    rng = np.random.default_rng(seed)
    parts = []
    for l, (ws, bs) in enumerate(layer_shapes()):
        fan_in = 9 * ws[1]
        w = rng.standard_normal(ws) * np.sqrt(2.0 / fan_in)
        if l == LAYERS - 1:
            w *= 0.1
        parts.append(w.reshape(-1))
        parts.append(np.zeros(bs))
    return np.concatenate(parts).astype(np.float32)
