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
