"""The learned warm start of the CDMFT bath fit: an MLP trained on the device
by the engine's own kernels (forward, backward, Adam; BF16 weights, FP32
accumulation).  No counterpart in the reference, whose CDMFT starts from the
user's bath (or from its loop predictor, pyqcm/_loop.py:15-40).

Inputs and outputs are standardized with the training set's mean and
standard deviation; the network maps model parameters (U, mu, t', ...) to
converged bath parameters.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib, ptr


class MLP:
    """Device MLP with tanh hidden layers and a linear output layer."""

    def __init__(self, widths, seed=0):
        self.widths = [int(w) for w in widths]
        arr = (ctypes.c_int * len(self.widths))(*self.widths)
        h = ctypes.c_void_p()
        check(lib().qcmg_mlp_create(len(self.widths) - 1, arr, ctypes.byref(h)))
        self._h = h
        n = ctypes.c_size_t()
        check(lib().qcmg_mlp_num_params(self._h, ctypes.byref(n)))
        self.n_params = n.value
        self.set_params(self.initial_params(seed))
        self.x_mean = self.x_std = self.y_mean = self.y_std = None

    def __del__(self):
        if getattr(self, "_h", None):
            lib().qcmg_mlp_destroy(self._h)
            self._h = None

    def initial_params(self, seed):
        """Glorot-uniform weights, zero biases (seeded)."""
        rng = np.random.default_rng(seed)
        p = []
        for a, b in zip(self.widths[:-1], self.widths[1:]):
            lim = np.sqrt(6.0 / (a + b))
            p.append(rng.uniform(-lim, lim, a * b))
            p.append(np.zeros(b))
        return np.concatenate(p).astype(np.float32)

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        check(lib().qcmg_mlp_set_params(self._h, ptr(p)))

    def get_params(self):
        p = np.zeros(self.n_params, np.float32)
        check(lib().qcmg_mlp_get_params(self._h, ptr(p)))
        return p

    def forward_raw(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((x.shape[0], self.widths[-1]), np.float32)
        check(lib().qcmg_mlp_forward(self._h, x.shape[0], ptr(x), ptr(y)))
        return y

    def loss_grad_raw(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(self.n_params, np.float32)
        loss = ctypes.c_float()
        check(lib().qcmg_mlp_loss_grad(self._h, x.shape[0], ptr(x), ptr(t), ctypes.byref(loss),
                                       ptr(g)))
        return loss.value, g

    def train_raw(self, x, t, epochs, batch, lr, seed=0):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = ctypes.c_float()
        check(lib().qcmg_mlp_train(self._h, x.shape[0], ptr(x), ptr(t), int(epochs), int(batch),
                                   float(lr), int(seed), ctypes.byref(loss)))
        return loss.value

    # -- standardized interface
    def fit(self, X, Y, epochs=2000, batch=64, lr=1e-3, seed=0):
        X, Y = np.asarray(X, np.float64), np.asarray(Y, np.float64)
        self.x_mean, self.x_std = X.mean(0), X.std(0) + 1e-12
        self.y_mean, self.y_std = Y.mean(0), Y.std(0) + 1e-12
        return self.train_raw((X - self.x_mean) / self.x_std, (Y - self.y_mean) / self.y_std, epochs,
                              min(batch, len(X)), lr, seed)

    def predict(self, X):
        X = np.atleast_2d(np.asarray(X, np.float64))
        y = self.forward_raw((X - self.x_mean) / self.x_std).astype(np.float64)
        return y * self.y_std + self.y_mean
