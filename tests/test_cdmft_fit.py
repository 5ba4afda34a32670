"""The CDMFT bath fit on the host (no GPU): residuals and distance against the
reference's CDMFT_distance on its own host function (golden fixture), the
exact Jacobian against central differences, and a fit that lowers the
distance.  The host G_host(iw) of the golden case is the reference's."""
import numpy as np
import pytest

from conftest import load_golden
from lattice_helpers import build_lattice


@pytest.fixture(scope="module")
def case():
    g = load_golden("lat_cdmft2x2_b4")
    lm = build_lattice("lat_cdmft2x2_b4")
    wn = np.array([(2 * n + 1) * np.pi / 50.0 for n in range(20)])
    return g, lm, wn


def _fit(case, names):
    from pyqcm_gb300.cdmft import BathFit
    g, lm, wn = case
    values = lm.cluster_values()
    return BathFit(lm.cluster, values, names, wn, np.ones_like(wn), g["host"])


def test_distance_matches_reference(case):
    g, lm, wn = case
    fit = _fit(case, ["eb1", "eb2", "tb1"])
    for p, ref in (((-1.0, 1.0, 0.5), g["dist0"]), ((-1.2, 0.8, 0.45), g["dist1"])):
        d = fit.distance(np.array(p))
        assert abs(d - float(ref)) <= 1e-12 * max(1.0, abs(float(ref))), (d, float(ref))


def test_residuals_square_sum_is_the_distance(case):
    fit = _fit(case, ["eb1", "eb2", "tb1"])
    x = np.array([-1.1, 0.9, 0.55])
    r = fit.residuals(x)
    dw = 2 * np.pi / 50.0
    assert np.isclose(2 * np.sum(r ** 2) * dw / 16, fit.distance(x), rtol=1e-13)


def test_exact_jacobian_against_central_differences(case):
    names = ["eb1", "eb2", "eb3", "eb4", "tb1", "tb2", "tb3", "tb4"]
    fit = _fit(case, names)
    x = np.array([-1.0, 1.0, -0.6, 0.6, 0.5, 0.5, 0.4, 0.4])
    J = fit.jacobian(x)
    h = 1e-6
    for p in range(len(x)):
        e = np.zeros_like(x)
        e[p] = h
        fd = (fit.residuals(x + e) - fit.residuals(x - e)) / (2 * h)
        assert np.max(np.abs(J[:, p] - fd)) <= 1e-7 * max(1.0, np.max(np.abs(fd))), p
    # the accumulation used when a parameter hits one row twice gives the same
    fit.theta_unique = fit.E_unique = False
    assert np.allclose(fit.jacobian(x), J, rtol=0, atol=1e-14 * np.max(np.abs(J)))


def test_jacobian_with_a_nondiagonal_bath(case):
    """A bath-bath hopping makes E non-diagonal: the resolvent then comes
    from the full inverse; the Jacobian still matches central differences."""
    fit = _fit(case, ["eb1", "eb2", "tb1", "tb2"])
    fit.E0 = fit.E0.copy()
    fit.E0[0, 1] = fit.E0[1, 0] = 0.3
    x = np.array([-1.0, 1.0, 0.5, 0.4])
    J = fit.jacobian(x)
    h = 1e-6
    for p in range(len(x)):
        e = np.zeros_like(x)
        e[p] = h
        fd = (fit.residuals(x + e) - fit.residuals(x - e)) / (2 * h)
        assert np.max(np.abs(J[:, p] - fd)) <= 1e-7 * max(1.0, np.max(np.abs(fd))), p


def test_fit_lowers_the_distance(case):
    from pyqcm_gb300.cdmft import fit_bath
    names = ["eb1", "eb2", "eb3", "eb4", "tb1", "tb2", "tb3", "tb4"]
    fit = _fit(case, names)
    x0 = np.array([-1.0, 1.0, -0.6, 0.6, 0.5, 0.5, 0.4, 0.4])
    x, nfev = fit_bath(fit, x0)
    assert fit.distance(x) < fit.distance(x0)
    # near a stationary point of the least-squares cost (the reference's
    # tolerances stop on the step size, xtol = 1e-6)
    g0 = fit.jacobian(x0).T @ fit.residuals(x0)
    g = fit.jacobian(x).T @ fit.residuals(x)
    assert np.linalg.norm(g) < 1e-3 * np.linalg.norm(g0)


def test_convergence_manager_depth():
    from pyqcm_gb300.cdmft import ConvergenceManager
    c = ConvergenceManager(1e-4, depth=2)
    assert not c.test([1.0, 2.0])
    assert not c.test([1.0, 2.0])
    assert c.test([1.0, 2.0 + 1e-5])
    assert not c.test([1.5, 2.0])
