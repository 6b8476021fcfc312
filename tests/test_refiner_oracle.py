"""The refiner's FP64 oracle is itself checked by finite differences (CPU)."""
import numpy as np

import refiner_oracle as ro


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    theta = ro.init(5)
    x = rng.random((3, 81))
    t = rng.uniform(-0.5, 0.5, (3, 2))
    loss, g, _ = ro.loss_grad(theta, x, t)
    # the variance term's r^2 is a stop-gradient for the means: check that with
    # a loss built the same way
    def L(th):
        out, _ = ro.forward(th, x)
        r2 = (out[:, 0] - t[:, 0]) ** 2 + (out[:, 1] - t[:, 1]) ** 2
        return np.mean(0.5 * r2 + out[:, 2])   # the means and the s-linear part
    idx = rng.choice(ro.NPARAM, 40, replace=False)
    out0, _ = ro.forward(theta, x)
    r2_0 = (out0[:, 0] - t[:, 0]) ** 2 + (out0[:, 1] - t[:, 1]) ** 2
    def L_full(th):
        out, _ = ro.forward(th, x)
        r2 = (out[:, 0] - t[:, 0]) ** 2 + (out[:, 1] - t[:, 1]) ** 2
        return np.mean(0.5 * r2 + 0.5 * r2_0 * np.exp(-out[:, 2]) + out[:, 2])
    for i in idx:
        e = np.zeros_like(theta); e[i] = 1e-6
        fd = (L_full(theta + e) - L_full(theta - e)) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])
    assert ro.NPARAM == 37507
