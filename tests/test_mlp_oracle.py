"""The MLP oracle on the CPU: its backpropagated gradient against central
differences (FP64, no weight rounding), and its BF16 rounding."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle as mo  # noqa: E402


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5], np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # halfway rounds to the even mantissa
    assert r[2] == np.float32(1.0 + 4 * 2 ** -8)
    assert r[3] == 1.0 and r[4] == -2.5


def test_gradient_against_central_differences():
    rng = np.random.default_rng(3)
    widths = [4, 7, 6, 3]
    n = sum(a * b + b for a, b in zip(widths[:-1], widths[1:]))
    p = rng.normal(0, 0.5, n)
    x = rng.normal(size=(9, 4))
    t = rng.normal(size=(9, 3))
    loss, g = mo.loss_grad(widths, p, x, t, rounding=False)
    h = 1e-6
    for k in rng.choice(n, 25, replace=False):
        e = np.zeros(n)
        e[k] = h
        fd = (mo.loss_grad(widths, p + e, x, t, False)[0] - mo.loss_grad(widths, p - e, x, t, False)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-7 * max(1.0, abs(fd)), (k, fd, g[k])
