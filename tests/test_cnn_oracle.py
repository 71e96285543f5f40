"""The CPU oracle of the warm-start network checks itself: its analytic
gradients against central finite differences of its own loss (with the BF16
operand rounding switched off, so the loss is smooth)."""

import numpy as np

import cnn_oracle as CO


def test_oracle_unet_gradient_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(CO, "bf16", lambda x: np.asarray(x, np.float64))
    net = CO.UNet(height=8, in_channels=2, base_channels=8, levels=3)
    rng = np.random.default_rng(0)
    theta = rng.normal(0, 0.3, net.nparams)
    x = rng.normal(0, 1, (2, 2, 8, 8))
    t = rng.normal(0, 1, (2, 1, 8, 8))
    loss, g, _ = net.loss_grad(theta, x, t)
    idx = rng.choice(net.nparams, 40, replace=False)
    h = 1e-6
    for i in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        fd = (net.loss_grad(tp, x, t)[0] - net.loss_grad(tm, x, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -9, -2.5], np.float32)
    r = CO.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0  # a tie rounds to the even neighbour
    assert r[2] == 1.0 + 2 ** -7  # above half an ulp
    assert r[3] == 1.0  # below half an ulp
    assert r[4] == -2.5
