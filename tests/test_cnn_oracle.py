"""The CPU reference of the learned update network (no GPU): its analytic
gradient matches central finite differences in FP64, and its BF16 rounding
matches round-to-nearest-even."""
import numpy as np

import cnn_oracle as K


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -2.5, 3.0e-3], np.float32)
    r = K.bf16(x)
    # bf16 keeps 7 mantissa bits: spacing 2^-7 at 1
    assert r[0] == 1.0
    assert r[1] == 1.0                      # exactly half way: ties to even
    assert r[2] == 1.0                      # below half way
    assert r[3] == 1.0 + 2 ** -7            # above half way
    assert r[4] == -2.5
    assert abs(r[5] - 3.0e-3) / 3.0e-3 < 2 ** -8


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    B, H, W = 1, 5, 6
    p = 0.3 * rng.standard_normal(K.N_PARAMS)
    feat = rng.standard_normal((B, 3, H, W))
    tgt = rng.standard_normal((B, H, W))
    mask = (rng.random((B, H, W)) > 0.3).astype(np.float64)
    loss, g = K.loss_and_grad(p, feat, tgt, mask, emulate=False)
    offs = {name: 0 for name, _ in K.SHAPES}
    o = 0
    for name, shp in K.SHAPES:
        offs[name] = o
        o += int(np.prod(shp))
    picks = [offs["W1"] + 5, offs["W2"] + 1234, offs["W3"] + 77, offs["W4"] + 4000, offs["b4"] + 3,
             offs["W5"] + 100, offs["b5"], offs["b1"] + 7]
    h = 1e-6
    for i in picks:
        e = np.zeros_like(p)
        e[i] = h
        fd = (K.loss_and_grad(p + e, feat, tgt, mask, emulate=False)[0] -
              K.loss_and_grad(p - e, feat, tgt, mask, emulate=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])
