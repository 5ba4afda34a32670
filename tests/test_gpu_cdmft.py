"""The CDMFT loop on the GPU: impurity solve and host function on the device,
bath fit on the host, fixed-point iteration to the 'parameters' test."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import pyqcm_gb300
    pyqcm_gb300.lib()
    return pyqcm_gb300


def _loop(lm, x0=None, maxiter=60):
    from pyqcm_gb300.cdmft import CDMFT
    names = ["eb1_1", "eb2_1", "eb3_1", "eb4_1", "tb1_1", "tb2_1", "tb3_1", "tb4_1"]
    c = CDMFT(lm, names, grid=(39 * np.pi / 50, 50.0), kside=8, maxiter=maxiter, x0=x0)
    return c, c.run()


def test_cdmft_converges_to_a_fixed_point(pg):
    from lattice_helpers import build_lattice
    lm = build_lattice("lat_cdmft2x2_b4")
    c, x = _loop(lm)
    assert np.all(np.isfinite(x))
    assert c.niter >= 3
    # converged: one more step from the solution reproduces it
    x2 = c.step(x)
    assert np.linalg.norm(x2 - x) / len(x) < 1e-3, (x, x2)


def test_cdmft_same_solution_from_a_perturbed_start(pg):
    from lattice_helpers import build_lattice
    lm = build_lattice("lat_cdmft2x2_b4")
    c1, x1 = _loop(lm)
    lm2 = build_lattice("lat_cdmft2x2_b4")
    c2, x2 = _loop(lm2, x0=x1 + 0.02 * np.array([1, -1, 1, -1, 1, 1, -1, -1]))
    # same fixed point (up to the order of equivalent bath orbitals)
    e1, t1 = np.sort(x1[:4]), np.sort(np.abs(x1[4:]))
    e2, t2 = np.sort(x2[:4]), np.sort(np.abs(x2[4:]))
    assert np.max(np.abs(e1 - e2)) < 1e-3 and np.max(np.abs(t1 - t2)) < 1e-3, (x1, x2)


def test_concurrent_loops_match_sequential_runs(pg):
    """Two loops in flight at once (run_many, one host thread each, separate
    device handles and streams) converge to the same baths as the same loops
    run one after the other: the engine's reductions are deterministic, so
    the results agree to rounding."""
    from lattice_helpers import build_lattice
    from pyqcm_gb300.cdmft import CDMFT, run_many
    names = ["eb1_1", "eb2_1", "eb3_1", "eb4_1", "tb1_1", "tb2_1", "tb3_1", "tb4_1"]

    def loops():
        out = []
        for U in (4.0, 6.0):
            lm = build_lattice("lat_cdmft2x2_b4")
            lm.set_parameters(dict(lm.params, U=U, mu=U / 2))
            out.append(CDMFT(lm, names, grid=(39 * np.pi / 50, 50.0), kside=8, maxiter=60))
        return out

    seq = run_many(loops(), workers=1)
    par = run_many(loops(), workers=2)
    for (xs, _, es), (xp, _, ep) in zip(seq, par):
        assert es is None and ep is None, (es, ep)
        assert np.max(np.abs(xs - xp)) < 1e-12, (xs, xp)


def _converged_host_fit(fit, x0):
    """SciPy's 'trf' fit of the residuals, then exact Gauss-Newton steps until
    the gradient J^T r stops decreasing.  The solver's cost-based tests stop
    once the remaining decrease is below the cost's rounding, which on these
    large-residual fits leaves a gradient of ~1e-8 and the bath determined to
    ~1e-8 only; the polish brings the gradient to ~1e-13."""
    import scipy.optimize
    x = scipy.optimize.least_squares(fit.residuals, x0, jac=fit.jacobian, method="trf",
                                     ftol=1e-15, xtol=1e-15, gtol=1e-15, max_nfev=5000).x
    grad = lambda v: np.max(np.abs(fit.jacobian(v).T @ fit.residuals(v)))
    best = grad(x)
    for _ in range(200):
        J, r = fit.jacobian(x), fit.residuals(x)
        xn = x - np.linalg.solve(J.T @ J, J.T @ r)
        gn = grad(xn)
        if gn >= best:
            break
        x, best = xn, gn
    return x, best


@pytest.mark.parametrize("case", ["b4", "b8x16"])
def test_device_bath_fit_reproduces_the_host_fit(pg, case):
    """The device bath fit (qcmg_bath_fit, Levenberg-Marquardt on the exact
    normal equations, one CTA per instance, three instances in one call)
    reaches the bath of the host fit of the same residuals to 1e-8, on the
    reference's own host functions: the 4-bath golden case (20 frequencies)
    and the 8-bath, 16-hybridization case at its benchmarked grids (200
    frequencies, 64x64 k).  The host fit is SciPy's 'trf' converged to a
    gradient of ~1e-13 (_converged_host_fit).

    The fits have several local minima (the 4-bath plaquette's bath energies
    have wells at +-0.63) and the solvers' paths differ, so the device starts
    at three points near the host's minimum.  From the model's own start the
    device fit must reach a local minimum of the same residuals."""
    from conftest import GOLDEN, load_golden
    from pyqcm_gb300.cdmft import BathFit, fit_bath_device
    if case == "b4":
        from lattice_helpers import build_lattice
        g = load_golden("lat_cdmft2x2_b4")
        lm = build_lattice("lat_cdmft2x2_b4")
        wn = np.array([(2 * n + 1) * np.pi / 50.0 for n in range(20)])
        names = ["eb1", "eb2", "eb3", "eb4", "tb1", "tb2", "tb3", "tb4"]
    else:
        import sys
        sys.path.insert(0, GOLDEN)
        from make_golden import BENCH_C4_PARAMS
        from pyqcm_gb300.cdmft import plaquette_bath_model
        g = load_golden("bench_cdmft2x2_b8")
        lm = plaquette_bath_model(8, "R0:N12:S0", hybridizations=2)
        lm.set_parameters(dict(BENCH_C4_PARAMS))
        wn = g["host_w"]
        names = [f"eb{k+1}" for k in range(8)] + [f"tb{k+1}" for k in range(16)]
    lm.finalize()
    fit = BathFit(lm.cluster, lm.cluster_values(), names, wn, np.ones_like(wn), g["host"])
    x0 = np.array([lm.cluster_values()[n] for n in names])
    xh, gh = _converged_host_fit(fit, x0)
    assert gh < 1e-11, gh
    ch = 0.5 * np.sum(fit.residuals(xh) ** 2)
    rng = np.random.default_rng(7)
    starts = [xh + 1e-3 * rng.standard_normal(len(xh)) for _ in range(3)]
    xd, cost, it, st = fit_bath_device([fit] * 3, starts, accur_bath=1e-15, accur_dist=0.0,
                                       gtol=1e-12, max_iter=1000)
    for k in range(3):
        assert np.all(np.isfinite(xd[k])) and st[k] in (2, 3), (k, st[k], it[k])
        assert np.max(np.abs(xd[k] - xh)) < 1e-8, (k, np.max(np.abs(xd[k] - xh)), it[k], st[k])
        assert abs(cost[k] - ch) < 1e-13 * ch, (k, cost[k], ch)
        assert abs(cost[k] - 0.5 * np.sum(fit.residuals(xd[k]) ** 2)) < 1e-12 * cost[k]
    # from the model's start: a local minimum of the same residuals
    x1, c1, _, s1 = fit_bath_device([fit], [x0], accur_bath=1e-15, accur_dist=0.0, gtol=1e-12,
                                    max_iter=1000)
    grad = fit.jacobian(x1[0]).T @ fit.residuals(x1[0])
    assert np.max(np.abs(grad)) < 1e-9, (s1, np.max(np.abs(grad)))


def test_batched_loops_match_sequential_runs(pg):
    """run_batched (every loop's impurity ground states in one graph-replayed
    lanczos_batch, every bath fit in one qcmg_bath_fit launch) reaches the
    same baths as the loops run one by one (run_many with one worker): the
    batched ground states are bitwise those of the host-driven recurrence and
    the fits run the same per-instance code."""
    from lattice_helpers import build_lattice
    from pyqcm_gb300.cdmft import CDMFT, run_batched, run_many
    names = ["eb1_1", "eb2_1", "eb3_1", "eb4_1", "tb1_1", "tb2_1", "tb3_1", "tb4_1"]

    def loops():
        out = []
        for U in (3.0, 4.0, 6.0):
            lm = build_lattice("lat_cdmft2x2_b4")
            lm.set_parameters(dict(lm.params, U=U, mu=U / 2))
            out.append(CDMFT(lm, names, grid=(39 * np.pi / 50, 50.0), kside=8, maxiter=60))
        return out

    seq = run_many(loops(), workers=1)
    ls = loops()
    bat = run_batched(ls, workers=3)
    for (xs, _, es), (xb, _, eb), c in zip(seq, bat, ls):
        assert es is None and eb is None, (es, eb)
        assert np.array_equal(xs, xb), (xs, xb)
        assert c.niter >= 3


def test_batched_groups_match_one_group(pg):
    """Two lockstep groups in their own threads reach the same baths as one."""
    from lattice_helpers import build_lattice
    from pyqcm_gb300.cdmft import CDMFT, run_batched
    names = ["eb1_1", "eb2_1", "eb3_1", "eb4_1", "tb1_1", "tb2_1", "tb3_1", "tb4_1"]

    def loops():
        out = []
        for U in (3.0, 4.0, 5.0, 6.0):
            lm = build_lattice("lat_cdmft2x2_b4")
            lm.set_parameters(dict(lm.params, U=U, mu=U / 2))
            out.append(CDMFT(lm, names, grid=(39 * np.pi / 50, 50.0), kside=8, maxiter=60))
        return out

    one = run_batched(loops(), workers=4, groups=1)
    two = run_batched(loops(), workers=4, groups=2)
    for (x1, _, e1), (x2, _, e2) in zip(one, two):
        assert e1 is None and e2 is None, (e1, e2)
        assert np.array_equal(x1, x2)


def _reference_loop():
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "cdmft_loop_b4.npz"))


def test_fixed_point_loop_matches_the_reference_loop(pg):
    """The whole CDMFT loop against the reference's own: the 4-bath plaquette
    iterated with the fixed point to the 'parameters' test (depth 2, accur
    1e-8), each step's bath fitted tightly (xtol 1e-12, ftol 1e-15; loose
    fits stop at different points of the distance's flat directions, 1e-6
    apart) -- tests/golden/make_cdmft_loop.py ran the reference's C++ host
    function, residuals and gradient under SciPy's trf.  With the host fit
    (trf on the engine's residuals and exact Jacobian): the same number of
    steps, every iterate and the converged bath within 1e-7 of the
    reference's, most iterates within 1e-9.  The distance fixes the bath
    only to ~1e-8 in its softest directions (a displacement d there changes
    the cost by ~d^2 times a small curvature, below the cost's rounding), so
    two exact fits with different Jacobians (exact here, finite differences
    in the reference) stop up to a few 1e-8 apart."""
    from lattice_helpers import build_lattice
    from pyqcm_gb300.cdmft import CDMFT
    g = _reference_loop()
    names = [str(v) for v in g["varia"]]
    lm = build_lattice("lat_cdmft2x2_b4")
    c = CDMFT(lm, names, grid=(39 * np.pi / 50, 50.0), kside=8, maxiter=int(g["maxiter"]),
              depth=int(g["depth"]), accur=float(g["accur"]), accur_bath=float(g["accur_bath"]),
              accur_dist=float(g["accur_dist"]), iteration="fixed_point", fit="host")
    x = c.run()
    hist = np.array(c.history)
    ref = g["history"][1:]
    assert c.niter == int(g["iterations"]), (c.niter, int(g["iterations"]))
    assert np.max(np.abs(hist - ref)) < 1e-7, np.max(np.abs(hist - ref), axis=1)
    assert np.median(np.max(np.abs(hist - ref), axis=1)) < 1e-9
    assert np.max(np.abs(x - g["x"])) < 1e-7, (x, g["x"])


def test_fixed_point_loop_with_the_device_fit(pg):
    """The same loop with the device bath fit (Levenberg-Marquardt on the
    normal equations, finished by Gauss-Newton steps on the gradient).  From
    the loop's default start the two optimizers can end in different local
    minima of the first fit (the plaquette's bath has mirror minima with the
    energies of a pair of bath orbitals exchanged in sign: SciPy's trf crosses
    to eb1 = +0.635, the damped steps stay at -0.616), so this loop starts
    from the reference's first fitted bath.  Its fits carry ~1e-8 of the
    normal equations' rounding, so it runs to the parameters test at 1e-7:
    its first step within 1e-7 of the reference's second, its converged bath
    within 1e-6 of the reference's."""
    from lattice_helpers import build_lattice
    from pyqcm_gb300.cdmft import CDMFT
    g = _reference_loop()
    names = [str(v) for v in g["varia"]]
    lm = build_lattice("lat_cdmft2x2_b4")
    ref = g["history"]
    c = CDMFT(lm, names, grid=(39 * np.pi / 50, 50.0), kside=8, maxiter=int(g["maxiter"]),
              depth=int(g["depth"]), accur=1e-7, accur_bath=float(g["accur_bath"]),
              accur_dist=0.0, iteration="fixed_point", fit="device", x0=ref[1].copy())
    x = c.run()
    hist = np.array(c.history)
    assert np.max(np.abs(hist[0] - ref[2])) < 1e-7, (hist[0], ref[2])
    assert np.max(np.abs(x - g["x"])) < 1e-6, (x, g["x"], c.niter)
