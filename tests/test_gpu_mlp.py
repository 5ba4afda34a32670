"""The warm-start MLP on the GPU against its CPU oracle (oracle/mlp_oracle.py):
forward pass and gradients with the BF16-rounded weights, and a training
run that fits a smooth map."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle as mo  # noqa: E402

pytestmark = pytest.mark.gpu

WIDTHS = [4, 256, 256, 24]  # the configs' warm-start network: 73,240 parameters


@pytest.fixture(scope="module")
def net():
    from pyqcm_gb300.mlp import MLP
    m = MLP(WIDTHS, seed=5)
    assert m.n_params == 73240
    return m


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, WIDTHS[0])).astype(np.float32)
    t = rng.normal(size=(n, WIDTHS[-1])).astype(np.float32)
    return x, t


def test_forward_matches_oracle(net):
    p = net.get_params()
    x, _ = _data(100, 1)
    y = net.forward_raw(x)
    ref = mo.forward(WIDTHS, p, x)[-1]
    assert np.max(np.abs(y - ref)) <= 1e-5 * max(1.0, np.max(np.abs(ref)))


def test_gradient_matches_oracle(net):
    p = net.get_params()
    x, t = _data(257, 2)  # a batch that is not a multiple of the tile
    loss, g = net.loss_grad_raw(x, t)
    lref, gref = mo.loss_grad(WIDTHS, p, x, t)
    assert abs(loss - lref) <= 1e-5 * lref
    assert np.max(np.abs(g - gref)) <= 1e-4 * np.max(np.abs(gref))
    for (W, b), (Wr, br) in zip(mo.unpack(WIDTHS, g), mo.unpack(WIDTHS, gref)):
        assert np.max(np.abs(W - Wr)) <= 1e-4 * np.max(np.abs(Wr)) + 1e-12


def test_training_fits_a_smooth_map():
    from pyqcm_gb300.mlp import MLP
    rng = np.random.default_rng(4)
    X = rng.uniform(-1, 1, size=(512, 4))
    Y = np.stack([np.sin(X @ rng.normal(size=4)) for _ in range(6)], axis=1)
    m = MLP([4, 64, 64, 6], seed=1)
    before = float(np.mean((m.forward_raw(X.astype(np.float32)) - Y) ** 2))
    m.fit(X, Y, epochs=300, batch=64, lr=3e-3)
    after = float(np.mean((m.predict(X) - Y) ** 2))
    assert after < 0.02 * before, (before, after)
