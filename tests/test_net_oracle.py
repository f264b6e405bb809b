"""The CPU restatement of the reconstruction net (oracle/net_oracle.py) is
itself checked here: its backward pass against central finite differences
(float64, roundings off), its bfloat16 rounding against known values, and the
Adam step against the textbook formula."""
import numpy as np
import pytest

import net_oracle as no


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0 + 2 ** -8 + 2 ** -9, -3.140625, 0.0, 65504.0], np.float32)
    r = no.bf16(x)
    # 1+2^-8 is a tie -> even (1.0); 1+2^-8+2^-9 rounds up to 1+2^-7
    assert r[0] == 1.0 and r[1] == 1.0 and r[3] == 1.0078125
    assert r[4] == -3.140625 and r[5] == 0.0 and r[6] == 65536.0
    u = no.bf16(np.random.default_rng(0).standard_normal(1000).astype(np.float32)).astype(np.float32).view(np.uint32)
    assert np.all((u & 0xFFFF) == 0)


def test_param_count():
    assert no.NET_PARAMS == 9 * (8 * 16 + 16 * 16 * 2 + 16 * 4) + 16 * 3 + 4 == 6388


@pytest.mark.parametrize("H,W", [(5, 7), (9, 4)])
def test_backward_matches_finite_differences(H, W):
    rng = np.random.default_rng(H * 100 + W)
    p = no.init_params(3).astype(np.float64)
    p += rng.standard_normal(p.size) * 0.05  # biases away from zero: no ReLU kinks at the probe points
    feat = rng.random((8, H, W))
    feat[6:] = 0
    tgt = rng.random((3, H, W))

    out, acts = no.forward(p, feat, rounding=False)
    _, _, d = no.loss_grad(out, tgt, 0.1, 0.5)
    # lam = 0.5 is folded into d; the label is piecewise constant in p
    g = no.backward(p, acts, d, rounding=False)
    idx = rng.choice(p.size, 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (loss_fd(p + e, feat, tgt) - loss_fd(p - e, feat, tgt)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def loss_fd(pv, feat, tgt):
    # forward() casts params to float32 for unpacking; finite differences
    # need float64 throughout, so run the layers here on float64 views
    layers = []
    o = 0
    for ws, bs in no.layer_shapes():
        nw = int(np.prod(ws))
        layers.append((pv[o:o + nw].reshape(ws), pv[o + nw:o + nw + bs[0]]))
        o += nw + bs[0]
    a = feat
    for l, (w, b) in enumerate(layers):
        pre = no.conv(a, w, b)
        a = np.maximum(pre, 0.0) if l < no.LAYERS - 1 else pre
    out = a.copy()
    out[:3] += feat[:3]
    diff = out[:3] - tgt
    n = out.shape[1] * out.shape[2]
    label = (np.abs(diff).max(0) < 0.1).astype(np.float64)
    z = out[3]
    return (diff ** 2).sum() / 3.0 / n + 0.5 * (np.logaddexp(0.0, z) - label * z).sum() / n


def test_adam_step():
    p = np.array([1.0, -2.0]); m = np.zeros(2); v = np.zeros(2); g = np.array([0.5, -0.25])
    p1, m1, v1 = no.adam(p, m, v, g, 1, 0.01)
    # first step moves every parameter by ~lr against its gradient's sign
    assert np.allclose(p1, p - 0.01 * np.sign(g), atol=1e-7)
    assert np.allclose(m1, 0.1 * g) and np.allclose(v1, 0.001 * g * g)
