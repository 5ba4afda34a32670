"""Learned warm start of the CDMFT loop: training data from converged CDMFT
solves, training of the device MLP, and the comparison of CDMFT runs started
from the default bath and from the network's prediction.

Model: the 2x2 plaquette with bath orbitals (cdmft.plaquette_bath_model),
t = 1; inputs (U, mu, t') on U in [4, 12], t' in [-0.4, 0] and mu in
[0.35 U, 0.5 U] (half filling and hole doping; the sector is fixed, so the
chemical potential stands in for the doping), plus the feature mu / U.
Outputs: the converged bath energies and |hybridizations| (the hybridization
function depends on the hybridizations' squares only).  The default start
is the plain method's: a fixed bath, the same for every point.
"""
import time

import numpy as np

from .cdmft import CDMFT, bath_names, plaquette_bath_model

SECTORS = {4: "R0:N8:S0", 8: "R0:N12:S0"}


def default_bath(nb):
    """The plain start: bath energies spread on [-1, 1], hybridizations 0.5."""
    return np.concatenate([np.linspace(-1.0, 1.0, nb), 0.5 * np.ones(nb)])


def sample_params(n, seed):
    """(U, mu, t') rows, seeded."""
    rng = np.random.default_rng(seed)
    U = rng.uniform(4.0, 12.0, n)
    tp = rng.uniform(-0.4, 0.0, n)
    mu = U * rng.uniform(0.35, 0.5, n)
    return np.stack([U, mu, tp], axis=1)


def features(P):
    P = np.atleast_2d(np.asarray(P, np.float64))
    return np.concatenate([P, (P[:, 1] / P[:, 0])[:, None]], axis=1)


def canonical(x, nb):
    x = np.array(x, np.float64)
    x[nb:] = np.abs(x[nb:])
    return x


def solve(prow, x0, nb=4, kside=64, maxiter=64):
    """One CDMFT run from bath x0: (converged bath, iterations, seconds)."""
    U, mu, tp = (float(v) for v in prow)
    names = bath_names(nb)
    lm = plaquette_bath_model(nb, SECTORS[nb])
    params = {"t": 1.0, "tp": tp, "U": U, "mu": mu}
    params.update({k: float(v) for k, v in zip(names, x0)})
    lm.set_parameters(params)
    c = CDMFT(lm, names, grid=(399 * np.pi / 50, 50.0), kside=kside, maxiter=maxiter)
    t0 = time.perf_counter()
    x = c.run()
    return canonical(x, nb), c.niter, time.perf_counter() - t0


def generate(n, seed, nb=4, kside=64):
    """Converged baths from the default start for n seeded points: (P, Y,
    iterations, seconds); points whose loop fails are dropped."""
    P, Y, its, ts = [], [], [], []
    for prow in sample_params(n, seed):
        try:
            x, it, dt = solve(prow, default_bath(nb), nb, kside)
        except Exception:  # a point without a converged answer has no label
            continue
        P.append(prow)
        Y.append(x)
        its.append(it)
        ts.append(dt)
    return np.array(P), np.array(Y), np.array(its), np.array(ts)


def train(P, Y, hidden=(256, 256), epochs=3000, batch=64, lr=1e-3, seed=0):
    """The device MLP fitted to (features(P), Y)."""
    from .mlp import MLP
    X = features(P)
    m = MLP([X.shape[1], *hidden, Y.shape[1]], seed=seed)
    loss = m.fit(X, Y, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return m, loss


def save(path, P, Y, its, ts, seed, nb):
    np.savez_compressed(path, P=P, Y=Y, iterations=its, seconds=ts, seed=seed, n_bath=nb)


def load(path):
    d = np.load(path)
    return d["P"], d["Y"]


def evaluate(mlp, P, nb=4, kside=64):
    """For each point: CDMFT from the default start and from the network's
    prediction (falling back to the default start if that run fails).
    Returns a list of dicts."""
    out = []
    preds = mlp.predict(features(P))
    for prow, pred in zip(P, preds):
        xp, itp, tpl = solve(prow, default_bath(nb), nb, kside)
        fallback = False
        t0 = time.perf_counter()
        try:
            xw, itw, _ = solve(prow, canonical(pred, nb), nb, kside)
        except Exception:  # the plain start is the fallback
            fallback = True
            xw, itw, _ = solve(prow, default_bath(nb), nb, kside)
        tw = time.perf_counter() - t0
        out.append({"iters_plain": itp, "iters_warm": itw, "s_plain": tpl, "s_warm": tw,
                    "max_dx": float(np.max(np.abs(xw - xp))), "fallback": fallback,
                    "pred_err": float(np.max(np.abs(canonical(pred, nb) - xp)))})
    return out


if __name__ == "__main__":
    # python -m pyqcm_gb300.warmstart --n 224 --seed 1 --bath 4 --out FILE
    # generates a training set (needs a GPU)
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=224)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--bath", type=int, default=4, choices=[4, 8])
    ap.add_argument("--out", required=True)
    a = ap.parse_args()
    P, Y, its, ts = generate(a.n, a.seed, a.bath)
    save(a.out, P, Y, its, ts, a.seed, a.bath)
    print(f"{len(P)} of {a.n} points, mean iterations {its.mean():.2f}, mean {ts.mean():.2f} s")
