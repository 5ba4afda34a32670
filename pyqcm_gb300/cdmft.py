"""CDMFT self-consistency on the engine.

Restates the reference's CDMFT procedure (pyqcm/cdmft.py):
- the Matsubara frequency grid (frequency_grid('matsubara'), cdmft.py:846-851
  and :869, CDMFT weights 1);
- the 'parameters' convergence test of depth 2 (convergence_manager,
  cdmft.py:14-106);
- one CDMFT step (CDMFT_step, cdmft.py:479-628): solve the impurity problem
  (ground state + Green function on the device), build the host function
  G_host(iw) on the k grid (device), then fit the bath parameters so that the
  hybridization function matches -G_host;
- the bath fit by least squares on the residuals
  r_n = sqrt(w_n) (Gamma(iw_n) + G_host(iw_n)), real and imaginary parts
  (CDMFT_residuals, src_qcm/CPT.cpp:556-610), with the reference's
  tolerances (optimize(method='trf'), cdmft.py:1539-1640): on the device
  (qcmg_bath_fit, Levenberg-Marquardt on the exact normal equations) for a
  diagonal bath, else with scipy's 'trf' solver;
- the outer fixed-point iteration with damping (fixed_point_iteration,
  pyqcm/__init__.py:2773-2845).

Differences: the Jacobian of the residuals is exact (Gamma = theta (z - E)^-1
theta^T is linear in the bath parameters through theta and E) instead of the
reference's central differences (CPT.cpp:616-672), and the residuals are
stacked row-major per frequency (the reference's matrix storage order);
neither changes the least-squares optimum.
"""
import time

import numpy as np

from . import lattice as lat
from .ed import ClusterModel


def matsubara_grid(wc, beta):
    """(frequencies, integration weights, CDMFT weights) of the Matsubara grid
    up to wc at inverse temperature beta (cdmft.py:846-851, :869)."""
    wr = np.arange(np.pi / beta, wc + 1e-6, 2 * np.pi / beta)
    return wr, (2 * np.pi / beta) * np.ones_like(wr), np.ones_like(wr)


class ConvergenceManager:
    """The 'parameters' test: converged when |x - x_k| / n < tol for each of
    the depth previous iterates (cdmft.py:14-106)."""

    def __init__(self, tol, depth=2):
        self.tol, self.depth = tol, depth
        self.X = []

    def test(self, x):
        x = np.array(x, np.float64)
        if len(self.X) < self.depth:
            self.X.append(x)
            return False
        ok = all(np.linalg.norm(x - y) / x.shape[0] <= self.tol for y in self.X)
        self.X = self.X[1:] + [x]
        return ok


class BathFit:
    """Residuals of the bath fit and their exact Jacobian, for the cluster
    parameters `names` (cluster names: 'eb1', 'tb1', ...) of cluster model cm
    at fixed other parameter values `values`."""

    def __init__(self, cm, values, names, freqs, weights, host, spin_down=False):
        self.ns = cm.n_sites
        self.names = list(names)
        fixed = {k: v for k, v in values.items() if k not in self.names}
        T0 = cm.one_body_matrix(fixed, spin_down)
        self.theta0, self.E0 = T0[:self.ns, self.ns:], T0[self.ns:, self.ns:]
        self.dtheta, self.dE = [], []
        for n in self.names:  # the blocks are linear in each parameter
            Tp = cm.one_body_matrix({n: 1.0}, spin_down)
            self.dtheta.append(Tp[:self.ns, self.ns:])
            self.dE.append(Tp[self.ns:, self.ns:])
        # each parameter enters theta and E through a few entries only:
        # (parameter, row, column, value) of every nonzero entry
        def entries(mats):
            out = [(p, r, c, m[r, c]) for p, m in enumerate(mats) for r, c in zip(*np.nonzero(m))]
            cols = list(zip(*out)) if out else [(), (), (), ()]
            return (np.array(cols[0], np.intp), np.array(cols[1], np.intp),
                    np.array(cols[2], np.intp), np.array(cols[3], np.float64))
        self.nz_theta = entries(self.dtheta)
        self.nz_E = entries(self.dE)
        # fancy-index += is exact when no target repeats; np.add.at otherwise
        pa = set(zip(self.nz_theta[0].tolist(), self.nz_theta[1].tolist()))
        self.theta_unique = len(pa) == len(self.nz_theta[0])
        self.E_unique = len(set(self.nz_E[0].tolist())) == len(self.nz_E[0])
        self.iw = 1j * np.asarray(freqs, np.float64)
        self.sw = np.sqrt(np.asarray(weights, np.float64))
        self.host = np.asarray(host, np.complex128)
        self.nb = self.E0.shape[0]

    def diagonal_bath(self):
        """True when the bath has no bath-bath hopping (E diagonal for every
        parameter value): the form the device fit takes."""
        off = lambda m: np.count_nonzero(m - np.diag(np.diag(m)))
        return not off(self.E0) and not any(off(d) for d in self.dE)

    def blocks(self, x):
        th = self.theta0.copy()
        E = self.E0.copy()
        for xp, dth, dE in zip(x, self.dtheta, self.dE):
            th += xp * dth
            E += xp * dE
        return th, E

    def _sandwich(self, th, E):
        """(theta R, R theta^T) per frequency, R = (iw - E)^-1.  A diagonal
        bath (the usual case: bath energies only) needs no inverse."""
        if not np.count_nonzero(E - np.diag(np.diag(E))):
            r = 1.0 / (self.iw[:, None] - np.diag(E)[None, :])      # (nw, nb)
            thR = th[None, :, :] * r[:, None, :]
            return thR, thR.transpose(0, 2, 1)
        eye = np.eye(self.nb)
        R = np.linalg.inv(self.iw[:, None, None] * eye[None] - E[None])
        return th[None] @ R, R @ th.T[None]

    def gamma(self, x):
        th, E = self.blocks(x)
        thR, _ = self._sandwich(th, E)
        return thR @ th.T[None]

    def _pack(self, Z):
        Z = self.sw[:, None, None] * Z
        return np.concatenate([Z.real.reshape(len(Z), -1), Z.imag.reshape(len(Z), -1)], axis=1).ravel()

    def residuals(self, x):
        return self._pack(self.gamma(x) + self.host)

    def jacobian(self, x):
        th, E = self.blocks(x)
        thR, RthT = self._sandwich(th, E)   # (nw, ns, nb), (nw, nb, ns)
        # d_p = dth_p R th^T + th R dth_p^T + th R dE_p R th^T, from the few
        # nonzero entries of dth_p and dE_p (no small dense products)
        n, nw, ns = len(self.names), thR.shape[0], self.ns
        d = np.zeros((n, nw, ns, ns), np.complex128)
        P, A, B, V = self.nz_theta
        if len(P):
            t1 = V[:, None, None] * RthT[:, B, :].transpose(1, 0, 2)    # (nnz, w, c)
            t2 = V[:, None, None] * thR[:, :, B].transpose(2, 0, 1)     # (nnz, w, a)
            if self.theta_unique:
                d[P, :, A, :] += t1
                d[P, :, :, A] += t2
            else:
                np.add.at(d, (P, slice(None), A, slice(None)), t1)
                np.add.at(d, (P, slice(None), slice(None), A), t2)
        P, B, E3, V = self.nz_E
        if len(P):
            t3 = (V[:, None, None, None] * thR[:, :, B].transpose(2, 0, 1)[:, :, :, None]
                  * RthT[:, E3, :].transpose(1, 0, 2)[:, :, None, :])
            if self.E_unique:
                d[P] += t3
            else:
                np.add.at(d, P, t3)
        d *= self.sw[None, :, None, None]
        cols = np.concatenate([d.real.reshape(n, d.shape[1], -1), d.imag.reshape(n, d.shape[1], -1)],
                              axis=2)
        return cols.reshape(n, -1).T

    def distance(self, x, normal=True):
        """sum_n w_n |Gamma + G_host|^2 (x2 normal mixing) dw / dim^2, the
        reference's reporting scale (CPT.cpp:519-555) with CDMFT weights."""
        Z = self.gamma(x) + self.host
        w = self.sw ** 2
        d = float(np.sum(w[:, None, None] * np.abs(Z) ** 2))
        if normal:
            d *= 2
        dw = float(self.iw[1].imag - self.iw[0].imag) if len(self.iw) > 1 else 1.0
        return d * dw / (self.ns * self.ns)


def fit_bath(fit, x0, accur_bath=1e-6, accur_dist=1e-8, max_nfev=2000):
    """scipy least_squares 'trf' with the reference's tolerances
    (optimize(method='trf'), cdmft.py:1588-1603)."""
    import scipy.optimize
    sol = scipy.optimize.least_squares(fit.residuals, np.asarray(x0, np.float64), jac=fit.jacobian,
                                       method="trf", max_nfev=max_nfev, ftol=accur_dist,
                                       xtol=accur_bath, gtol=1e-12)
    return sol.x, sol.nfev


def fit_bath_device(fits, x0s, accur_bath=1e-6, accur_dist=1e-8, gtol=1e-12, max_iter=200):
    """The bath fits of several instances at once on the device
    (qcmg_bath_fit: one CTA per instance runs Levenberg-Marquardt on the
    exact normal equations).  fits: BathFit objects sharing one parameter
    structure and frequency grid; x0s: their start vectors.  Returns
    (x (n, npar), cost (n,), iterations (n,), status (n,))."""
    from ._lib import check, lib, ptr
    f0 = fits[0]
    n = len(fits)
    P, A, B, V = f0.nz_theta
    PE, BE, CE, VE = f0.nz_E
    if not all(f.diagonal_bath() for f in fits):
        raise ValueError("the device bath fit takes a diagonal bath (bath energies only)")
    ent_par = np.ascontiguousarray(np.concatenate([P, PE]).astype(np.int32))
    ent_kind = np.ascontiguousarray(np.concatenate([np.zeros(len(P)), np.ones(len(PE))]).astype(np.int32))
    ent_i = np.ascontiguousarray(np.concatenate([A, BE]).astype(np.int32))
    ent_j = np.ascontiguousarray(np.concatenate([B, CE]).astype(np.int32))
    ent_v = np.ascontiguousarray(np.concatenate([V, VE]).astype(np.float64))
    w = np.ascontiguousarray(f0.iw.imag)
    wt = np.ascontiguousarray(f0.sw ** 2)
    host = np.ascontiguousarray(np.stack([f.host for f in fits]).astype(np.complex128))
    th0 = np.ascontiguousarray(np.stack([f.theta0 for f in fits]).astype(np.float64))
    e0 = np.ascontiguousarray(np.stack([np.diag(f.E0) for f in fits]).astype(np.float64))
    x = np.ascontiguousarray(np.array(x0s, np.float64).reshape(n, -1))
    npar = x.shape[1]
    cost = np.zeros(n)
    it = np.zeros(n, np.int32)
    st = np.zeros(n, np.int32)
    check(lib().qcmg_bath_fit(n, f0.ns, f0.nb, len(w), ptr(w), ptr(wt), ptr(host), npar,
                              len(ent_par), ptr(ent_par), ptr(ent_kind), ptr(ent_i), ptr(ent_j),
                              ptr(ent_v), ptr(th0), ptr(e0), ptr(x), max_iter, accur_bath,
                              accur_dist, gtol, ptr(cost), ptr(it), ptr(st)))
    return x, cost, it, st


class CDMFT:
    """The CDMFT loop on a lattice model (pyqcm.cdmft.CDMFT with
    iteration='fixed_point', convergence='parameters', method='trf').

    varia: lattice-level bath parameter names of cluster 1 ('eb1_1', ...).
    grid: (wc, beta) of the Matsubara grid.  kside: side of the k grid of the
    host function.  x0: starting bath parameters (default: the model's).
    fit: 'device' fits the bath with Levenberg-Marquardt on the GPU
    (qcmg_bath_fit); 'host' with SciPy's trf on the exact Jacobian, the
    reference's optimizer.  The distance can have several local minima, and
    from a start far from all of them the two optimizers may end in
    different ones (the damped steps tend to stay on the start's side); the
    loop then converges to a different fixed point."""

    def __init__(self, model, varia, grid=(399 * np.pi / 50, 50.0), kside=64, maxiter=32,
                 miniter=0, depth=2, accur=1e-4, accur_bath=1e-6, accur_dist=1e-8, damping=0.0,
                 max_nfev=2000, x0=None, iteration="broyden", verbose=False, fit="device"):
        if iteration not in ("broyden", "fixed_point"):
            raise ValueError("iteration must be 'broyden' or 'fixed_point'")
        if fit not in ("device", "host"):
            raise ValueError("fit must be 'device' (qcmg_bath_fit) or 'host' (SciPy)")
        self.fit = fit
        self.iteration = iteration
        self.model = model
        self.varia = list(varia)
        self.cnames = [v[:-2] if v.endswith("_1") else v for v in self.varia]
        self.wr, _, self.cw = matsubara_grid(*grid)
        self.kside = kside
        self.maxiter, self.miniter = maxiter, miniter
        self.conv = ConvergenceManager(accur, depth)
        self.accur_bath, self.accur_dist, self.max_nfev = accur_bath, accur_dist, max_nfev
        self.damping = damping
        self.verbose = verbose
        if x0 is None:
            x0 = [model.params[v] for v in self.varia]
        self.x = np.array(x0, np.float64)
        self.niter = 0
        self.dist = None
        self.history = []
        self.time_ed = self.time_fit = 0.0

    # -- one CDMFT step, in phases (run_batched runs each phase for many loops)
    def _prepare(self, x):
        """Sets the bath x on the model and makes the instance; returns the
        Hamiltonians of its impurity ground-state sectors."""
        params = dict(self.model.params)
        params.update({v: float(xv) for v, xv in zip(self.varia, x)})
        self.model.set_parameters(params)
        self._t0 = time.perf_counter()
        self._inst = self.model.instance()
        return self._inst.cluster.gs_hamiltonians()

    def _host_fits(self, solved=None):
        """Impurity ground state (from `solved` when given), Green function and
        host function; returns one BathFit per spin block."""
        inst = self._inst
        inst.cluster.ground_state(solved)
        host = inst.CDMFT_host(self.wr, self.cw, kside=self.kside)
        self._t1 = time.perf_counter()
        values = dict(inst.cluster.values)
        return [BathFit(self.model.cluster, values, self.cnames, self.wr, self.cw, H, sd)
                for sd, H in host.items()]

    def _fit_one(self, fit, x):
        if self.fit == "device" and fit.diagonal_bath():
            xs, _, _, _ = fit_bath_device([fit], [x], self.accur_bath, self.accur_dist,
                                          max_iter=max(1, self.max_nfev // 10))
            return xs[0]
        return fit_bath(fit, x, self.accur_bath, self.accur_dist, self.max_nfev)[0]

    def _finish(self, fits, newx):
        normal = not (self._inst.cluster.mixing & 4)
        self.dist = sum(f.distance(newx, normal) for f in fits)
        t2 = time.perf_counter()
        self.time_ed += self._t1 - self._t0
        self.time_fit += t2 - self._t1
        self.E0 = self._inst.cluster.E0
        return newx

    def step(self, x):
        """One CDMFT step from bath x: returns the fitted bath (the spin
        blocks' fits in turn, each starting from the previous one's bath)."""
        self._prepare(x)
        fits = self._host_fits()
        newx = np.array(x, np.float64)
        for fit in fits:
            newx = self._fit_one(fit, newx)
        return self._finish(fits, newx)

    def run(self):
        """Iterates to self-consistency (Broyden or fixed point, as the
        reference's CDMFT does) until the fitted bath passes the parameters
        test; returns the converged bath."""
        gen = self._iterate()
        x = next(gen)
        try:
            while True:
                x = gen.send(self.step(x))
        except StopIteration:
            pass
        return self._settle()

    def _settle(self):
        params = dict(self.model.params)
        params.update({v: float(xv) for v, xv in zip(self.varia, self.x)})
        self.model.set_parameters(params)
        return self.x

    def _iterate(self):
        """The outer iteration as a generator: yields the bath at which a CDMFT
        step is needed and receives the step's fitted bath."""
        if self.iteration == "broyden":
            yield from self._broyden()
        else:
            yield from self._fixed_point()

    def _record(self, xs):
        self.xs = xs
        self.history.append(xs.copy())

    def _fixed_point(self):
        """x <- step(x), damped (fixed_point_iteration, pyqcm/__init__.py:2773-2845)."""
        x0 = self.x.copy()
        it = 0
        while True:
            xs = yield x0
            self._record(xs)
            x = xs + self.damping * (x0 - xs)   # (alpha - 1) F(x0) + x0, F = x0 - step(x0)
            it += 1
            if self.verbose:
                print(f"CDMFT iteration {it}: |dx| = {np.linalg.norm(x - x0):.3g}, "
                      f"distance = {self.dist:.3g}")
            x0 = x
            if self.conv.test(xs) and it >= self.miniter:
                break
            if it > self.maxiter:
                raise RuntimeError(f"CDMFT did not converge in {self.maxiter} iterations")
        self.x = x0
        self.niter = it

    def _broyden(self):
        """Broyden's root search on F(x) = x - step(x) with the inverse-Jacobian
        update of pyqcm.broyden (pyqcm/__init__.py, broyden), initial inverse
        Jacobian (1 + damping) * identity; the parameters test runs on the
        fitted bath of each step."""
        n = len(self.x)
        I = (1.0 + self.damping) * np.eye(n)
        x = self.x.copy()
        xs = yield x
        self._record(xs)
        f0 = x - xs
        f = f0.copy()
        it = 0
        while True:
            dx = -I @ f
            if np.any(np.isnan(dx)):
                raise RuntimeError("NaN produced in the Broyden iteration")
            x = x + dx
            if self.verbose:
                print(f"CDMFT Broyden iteration {it + 1}: |dx| = {np.linalg.norm(dx):.3g}, "
                      f"distance = {self.dist:.3g}")
            if np.linalg.norm(dx) < 1e-6 and it >= self.miniter:
                self.conv.test(self.xs)
                break
            if self.conv.test(self.xs) and it >= self.miniter:
                break
            xs = yield x
            self._record(xs)
            f = x - xs
            df = f - f0
            f0 = f.copy()
            I += np.outer(dx - I @ df, dx) @ I / (dx @ (I @ df))
            it += 1
            if it > self.maxiter:
                raise RuntimeError(f"CDMFT did not converge in {self.maxiter} iterations")
        self.x = x
        self.niter = it + 1


def run_batched(loops, workers=8, chunk=16, groups=1):
    """Runs CDMFT loops in lockstep with their device work batched (see
    _lockstep).  groups > 1 splits the loops round-robin into that many
    lockstep groups driven from host threads of their own, so that one group's
    batched ground states run on the device while another group's Green
    functions, host functions and fits run (workers are shared out among the
    groups).  Returns [(x, seconds, error)] in the order of `loops`."""
    groups = max(1, min(groups, len(loops)))
    if groups == 1:
        return _lockstep(loops, workers, chunk)
    from concurrent.futures import ThreadPoolExecutor
    idx = [list(range(g, len(loops), groups)) for g in range(groups)]
    per = max(1, workers // groups)
    with ThreadPoolExecutor(max_workers=groups) as ex:
        futs = [ex.submit(_lockstep, [loops[i] for i in ix], per, chunk) for ix in idx]
        res = [f.result() for f in futs]
    out = [None] * len(loops)
    for ix, r in zip(idx, res):
        for i, v in zip(ix, r):
            out[i] = v
    return out


def _lockstep(loops, workers=8, chunk=16):
    """Runs CDMFT loops in lockstep, one step of every unfinished loop at a
    time, with the device work of each step batched across the loops:
      1. every loop's impurity ground states in one lanczos_batch call (each
         sector's Lanczos steps replayed from a captured CUDA graph, all
         sectors side by side);
      2. the Green and host functions of each loop, in host threads (their
         device work overlaps);
      3. every loop's bath fit in one qcmg_bath_fit launch (one CTA per loop),
         per spin block, when the loops share one bath structure and use the
         device fit (each loop's own fit otherwise);
      4. each loop's Broyden or fixed-point update.
    The loops' iterates are those of running them one by one (the ground
    states are bitwise the same on the FP64 path).  Returns [(x, seconds,
    error)] in the order of `loops`, like run_many."""
    from concurrent.futures import ThreadPoolExecutor
    from .ed import lanczos_batch
    t_start = time.perf_counter()
    n = len(loops)
    out = [None] * n
    gens, pending = {}, {}

    def fail(i, e):
        out[i] = (None, time.perf_counter() - t_start, e)
        pending.pop(i, None)

    for i, c in enumerate(loops):
        try:
            gens[i] = c._iterate()
            pending[i] = next(gens[i])
        except Exception as e:  # noqa: BLE001 - reported per loop
            fail(i, e)
    with ThreadPoolExecutor(max_workers=max(1, workers)) as ex:
        while pending:
            # 1. instances and their ground-state sectors, solved together
            hs = {}
            for i in list(pending):
                try:
                    hs[i] = loops[i]._prepare(pending[i])
                except Exception as e:  # noqa: BLE001
                    fail(i, e)
            allh = [h for i in pending for h in hs[i]]
            res = lanczos_batch(allh, want_psi=True, chunk=chunk, raise_errors=False)
            solved, k = {}, 0
            for i in list(pending):
                solved[i] = {}
                for h in hs[i]:
                    e0, psi, _, err = res[k]
                    k += 1
                    if err is not None and i in pending:
                        fail(i, err)
                    solved[i][h] = (e0, psi)
            # 2. Green and host functions per loop
            live = list(pending)
            futs = {i: ex.submit(loops[i]._host_fits, solved[i]) for i in live}
            fits = {}
            for i in live:
                try:
                    fits[i] = futs[i].result()
                except Exception as e:  # noqa: BLE001
                    fail(i, e)
            # 3. bath fits: one device launch per spin block for the loops
            #    that share the first loop's structure, the others one by one
            live = list(pending)
            newx = {i: np.array(pending[i], np.float64) for i in live}
            nblk = max((len(fits[i]) for i in live), default=0)
            for blk in range(nblk):
                dev = [i for i in live if loops[i].fit == "device" and len(fits[i]) > blk
                       and fits[i][blk].diagonal_bath()]
                if dev:
                    ref = fits[dev[0]][blk]
                    same = [i for i in dev if _same_structure(fits[i][blk], ref)]
                    c0 = loops[same[0]]
                    xs, _, _, _ = fit_bath_device([fits[i][blk] for i in same],
                                                  [newx[i] for i in same], c0.accur_bath,
                                                  c0.accur_dist,
                                                  max_iter=max(1, c0.max_nfev // 10))
                    for j, i in enumerate(same):
                        newx[i] = xs[j]
                    dev = [i for i in dev if i not in same]
                for i in live:
                    if len(fits[i]) > blk and (i in dev or loops[i].fit != "device"
                                               or not fits[i][blk].diagonal_bath()):
                        try:
                            newx[i] = loops[i]._fit_one(fits[i][blk], newx[i])
                        except Exception as e:  # noqa: BLE001
                            fail(i, e)
            # 4. the outer iterations
            for i in list(pending):
                c = loops[i]
                try:
                    xs = c._finish(fits[i], newx[i])
                    pending[i] = gens[i].send(xs)
                except StopIteration:
                    out[i] = (c._settle(), time.perf_counter() - t_start, None)
                    pending.pop(i)
                except Exception as e:  # noqa: BLE001
                    fail(i, e)
    return out


def _same_structure(a, b):
    """True when two BathFits share parameters, entries and frequency grid
    (one qcmg_bath_fit launch can take both)."""
    return (len(a.names) == len(b.names) and a.ns == b.ns and a.nb == b.nb
            and np.array_equal(a.iw, b.iw) and np.array_equal(a.sw, b.sw)
            and all(np.array_equal(x, y) for x, y in zip(a.nz_theta, b.nz_theta))
            and all(np.array_equal(x, y) for x, y in zip(a.nz_E, b.nz_E)))


def run_many(loops, workers=4):
    """Runs independent CDMFT loops concurrently, one host thread per loop in
    flight.  Each loop owns its lattice model and, through it, its device
    handles and CUDA streams; the library's calls release the GIL, so one
    loop's kernels and host waits overlap the others' impurity solves, host
    functions and bath fits.  Returns [(x, seconds, error)] in the order of
    `loops` (x None and error the exception when a loop failed)."""
    from concurrent.futures import ThreadPoolExecutor
    from . import lib
    lib()  # load the library before the threads start

    def one(c):
        t0 = time.perf_counter()
        try:
            x = c.run()
            return x, time.perf_counter() - t0, None
        except Exception as e:  # reported per loop; the others still run
            return None, time.perf_counter() - t0, e

    if workers <= 1:
        return [one(c) for c in loops]
    with ThreadPoolExecutor(max_workers=workers) as ex:
        return list(ex.map(one, loops))


def plaquette_bath_model(n_bath=8, sector="R0:N12:S0", hybridizations=1):
    """The 2x2 plaquette with n_bath bath orbitals on the square lattice, with
    lattice operators t (nearest neighbour), tp (diagonal), U and the built-in
    mu.  Bath k has energy eb{k+1} and hybridization tb{k+1} with site k % 4;
    with hybridizations=2 it also couples to site (k+1) % 4 through
    tb{k+1+n_bath} (8 energies + 16 hybridizations for 8 baths: the
    batched-CDMFT configuration)."""
    from .lattice import LatticeModel
    if hybridizations not in (1, 2):
        raise ValueError("hybridizations must be 1 or 2")
    ns, no = 4, 4 + n_bath
    cm = ClusterModel(ns, n_bath)
    for k in range(n_bath):
        b, s = ns + k, k % ns
        cm.new_operator(f"eb{k+1}", "one-body", [(b, b, 1.0), (b + no, b + no, 1.0)])
        cm.new_operator(f"tb{k+1}", "one-body", [(s, b, 1.0), (s + no, b + no, 1.0)])
        if hybridizations == 2:
            s2 = (k + 1) % ns
            cm.new_operator(f"tb{k+1+n_bath}", "one-body", [(s2, b, 1.0), (s2 + no, b + no, 1.0)])
    lm = LatticeModel(cm, [(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0)], [(2, 0, 0), (0, 2, 0)])
    lm.interaction_operator("U", 1.0)
    lm.hopping_operator("t", (1, 0, 0), -1.0)
    lm.hopping_operator("t", (0, 1, 0), -1.0)
    lm.hopping_operator("tp", (1, 1, 0), -1.0)
    lm.hopping_operator("tp", (-1, 1, 0), -1.0)
    lm.set_target_sectors(sector)
    return lm


def bath_names(n_bath, hybridizations=1):
    """Lattice-level names of the bath parameters of plaquette_bath_model."""
    return ([f"eb{k+1}_1" for k in range(n_bath)]
            + [f"tb{k+1}_1" for k in range(hybridizations * n_bath)])
