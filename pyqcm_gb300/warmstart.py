"""Learned warm start of the CDMFT loop: training data from converged CDMFT
solves, training of the device MLP, and the comparison of CDMFT runs started
from the default bath and from the network's prediction.

Model: the 2x2 plaquette with bath orbitals (cdmft.plaquette_bath_model),
t = 1; inputs (U, mu, t') on U in [4, 12], t' in [-0.4, 0] and mu in
[0.35 U, 0.5 U] (half filling and hole doping; the sector is fixed, so the
chemical potential stands in for the doping), plus the feature mu / U.
Outputs: the converged bath energies and hybridizations in a canonical sign
(the hybridization function is unchanged when all the hybridizations of one
bath orbital change sign): 4 baths with one hybridization each, or 8 baths
with two each (8 energies + 16 hybridizations).  The default start is the
plain method's: a fixed bath, the same for every point.

generate_batched / evaluate_batched run many CDMFT loops at once through the
lockstep driver (cdmft.run_batched).
"""
import time

import numpy as np

from .cdmft import CDMFT, bath_names, plaquette_bath_model

SECTORS = {4: "R0:N8:S0", 8: "R0:N12:S0"}


def n_hyb(nb):
    """Hybridizations per bath orbital of the warm-start models."""
    return 2 if nb == 8 else 1


def default_bath(nb):
    """The plain start: bath energies spread on [-1, 1], hybridizations 0.5
    (0.5 and 0.25 with two per bath orbital)."""
    h = [0.5 * np.ones(nb)] + ([0.25 * np.ones(nb)] if n_hyb(nb) == 2 else [])
    return np.concatenate([np.linspace(-1.0, 1.0, nb)] + h)


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
    """Signs fixed: bath orbital k's first hybridization made positive (its
    other one follows the same flip)."""
    x = np.array(x, np.float64)
    if n_hyb(nb) == 1:
        x[nb:] = np.abs(x[nb:])
        return x
    for k in range(nb):
        if x[nb + k] < 0:
            x[nb + k] = -x[nb + k]
            x[2 * nb + k] = -x[2 * nb + k]
    return x


def solve(prow, x0, nb=4, kside=64, maxiter=64):
    """One CDMFT run from bath x0: (converged bath, iterations, seconds)."""
    U, mu, tp = (float(v) for v in prow)
    names = bath_names(nb, n_hyb(nb))
    lm = plaquette_bath_model(nb, SECTORS[nb], hybridizations=n_hyb(nb))
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


def _loop(prow, x0, nb, kside, maxiter, accur, accur_bath=1e-6, accur_dist=1e-8):
    U, mu, tp = (float(v) for v in prow)
    names = bath_names(nb, n_hyb(nb))
    lm = plaquette_bath_model(nb, SECTORS[nb], hybridizations=n_hyb(nb))
    params = {"t": 1.0, "tp": tp, "U": U, "mu": mu}
    params.update({k: float(v) for k, v in zip(names, x0)})
    lm.set_parameters(params)
    return CDMFT(lm, names, grid=(399 * np.pi / 50, 50.0), kside=kside, maxiter=maxiter,
                 accur=accur, accur_bath=accur_bath, accur_dist=accur_dist)


def generate_batched(n, seed, nb=8, kside=64, maxiter=64, accur=1e-7, groups=4, workers=8):
    """Converged baths from the default start for n seeded points, all loops
    run at once (run_batched): (P, Y, iterations, total seconds); points whose
    loop fails are dropped."""
    from .cdmft import run_batched
    Ps = sample_params(n, seed)
    loops = [_loop(p, default_bath(nb), nb, kside, maxiter, accur) for p in Ps]
    t0 = time.perf_counter()
    res = run_batched(loops, workers=workers, groups=groups)
    dt = time.perf_counter() - t0
    keep = [k for k, (x, _, e) in enumerate(res) if e is None]
    P = Ps[keep]
    Y = np.array([canonical(res[k][0], nb) for k in keep])
    its = np.array([loops[k].niter for k in keep])
    return P, Y, its, dt


def evaluate_batched(mlp, P, nb=8, kside=64, maxiter=64, accur=1e-7, groups=4, workers=8,
                     accur_bath=1e-10, accur_dist=1e-12):
    """The held-out points run twice, all loops of a run at once
    (run_batched): from the default start and from the network's prediction
    (a point whose warm run fails is rerun from the default start, its time
    added).  Each step's bath fit is converged tightly (accur_bath,
    accur_dist), so that the two runs' answers can agree to 1e-6.  Returns a
    dict: wall times, iterations, fallbacks, the largest difference between
    the two runs' converged baths, prediction errors."""
    from .cdmft import run_batched
    preds = [canonical(p, nb) for p in mlp.predict(features(P))]
    tight = dict(accur_bath=accur_bath, accur_dist=accur_dist)
    plain = [_loop(p, default_bath(nb), nb, kside, maxiter, accur, **tight) for p in P]
    t0 = time.perf_counter()
    rp = run_batched(plain, workers=workers, groups=groups)
    t_plain = time.perf_counter() - t0
    warm = [_loop(p, x0, nb, kside, maxiter, accur, **tight) for p, x0 in zip(P, preds)]
    t0 = time.perf_counter()
    rw = run_batched(warm, workers=workers, groups=groups)
    failed = [k for k, (_, _, e) in enumerate(rw) if e is not None]
    redo = [_loop(P[k], default_bath(nb), nb, kside, maxiter, accur, **tight) for k in failed]
    rr = run_batched(redo, workers=workers, groups=groups) if redo else []
    t_warm = time.perf_counter() - t0
    for k, r in zip(failed, rr):
        rw[k] = r
        warm[k] = redo[failed.index(k)]
    both = [k for k in range(len(P)) if rp[k][2] is None and rw[k][2] is None]
    dx = [float(np.max(np.abs(canonical(rw[k][0], nb) - canonical(rp[k][0], nb)))) for k in both]
    perr = [float(np.max(np.abs(preds[k] - canonical(rp[k][0], nb)))) for k in both]
    return {"s_plain": t_plain, "s_warm": t_warm, "points": len(P), "both_converged": len(both),
            "plain_failed": sum(r[2] is not None for r in rp),
            "iters_plain": [plain[k].niter for k in both],
            "iters_warm": [warm[k].niter for k in both],
            "fallbacks": len(failed), "max_dx": dx, "pred_err": perr}


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
    # python -m pyqcm_gb300.warmstart --n 600 --seed 1 --bath 8 --out FILE
    # generates a training set (needs a GPU): all loops at once, lockstep
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=600)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--bath", type=int, default=8, choices=[4, 8])
    ap.add_argument("--accur", type=float, default=1e-7)
    ap.add_argument("--groups", type=int, default=4)
    ap.add_argument("--out", required=True)
    a = ap.parse_args()
    P, Y, its, dt = generate_batched(a.n, a.seed, a.bath, accur=a.accur, groups=a.groups)
    save(a.out, P, Y, its, np.full(len(P), dt / max(len(P), 1)), a.seed, a.bath)
    print(f"{len(P)} of {a.n} points, mean iterations {its.mean():.2f}, {dt:.1f} s in all")
