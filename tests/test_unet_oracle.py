"""The FP64 U-Net oracle against central finite differences (it has no
reference counterpart to be pinned to, so it is pinned to calculus)."""
import numpy as np

from oracle import unet_oracle as U

C_IN, C_OUT, WIDTHS = 3, 3, (2, 3, 4, 4)


def test_param_count_of_the_warm_start_net():
    assert U.param_count(16, 3, (32, 64, 128, 128)) > 1_000_000
    assert U.param_count(3, 3, (32, 64, 128, 128)) == 1209411


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    n = U.param_count(C_IN, C_OUT, WIDTHS)
    flat = rng.standard_normal(n) * 0.4
    x = rng.standard_normal((2, 8, 16, C_IN))
    t = rng.standard_normal((2, 8, 16, C_OUT))
    loss, _, g = U.loss_and_grads(flat, x, t, C_IN, C_OUT, WIDTHS)
    idx = rng.choice(n, 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros(n)
        e[i] = h
        lp = U.loss_and_grads(flat + e, x, t, C_IN, C_OUT, WIDTHS)[0]
        lm = U.loss_and_grads(flat - e, x, t, C_IN, C_OUT, WIDTHS)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])
