"""The CPU oracle of the lattice integrals (oracle/lattice_oracle.py) against
the reference's own lattice layer (tests/golden): the Potthoff functional of
the benchmarked 3x4 VCA case on its full 128x128 k x 256 frequency grid from
the reference's Q-matrices, and, on the small lattice cases, the CPT
periodized Green function, the Potthoff functional and the CDMFT host
function from the oracle's own cluster solve.  No GPU needed."""
import numpy as np
import pytest

from conftest import load_golden
from lattice_helpers import build_lattice
from models import LATTICE_CASES

import lattice_oracle as lo


def _lattice(tag):
    lm = build_lattice(tag)
    lm.finalize()
    return lm


def _cluster(lm):
    cm = lm.cluster
    vals = lm.cluster_values()
    spins = (False, True)
    tcs = {sd: lo.one_body_blocks(cm.operators, vals, cm.n_orb, cm.n_sites, sd) for sd in spins}
    if all(np.allclose(tcs[False][k], tcs[True][k]) for k in range(3)):
        spins = (False,)
    e0, Q = lo.cluster_lehmann(cm.operators, vals, cm.n_orb, cm.n_sites, lm.target_sectors,
                               spins)
    return e0, Q, tcs


def test_sef_on_the_benchmarked_grid_from_reference_qmatrices():
    import bench
    g = load_golden("bench_vca3x4")
    lm = bench._vca_3x4()
    lm.finalize()
    w, wt = g["sef_w"], g["sef_wt"]
    trace, diag = 0.0, 0.0
    for sd, q in ((False, "qup"), (True, "qdn")):
        R, els, hdiff, _ = lm.fourier(sd)
        B, ldg = lo.base([(g[q + "_e"], g[q + "_v"].T, 1.0)], np.zeros((12, 0)), np.zeros(0),
                         hdiff, 1j * w)
        trace += lo.sef_grid(B, ldg, wt, R, els, (128, 128, 1), nthreads=8)
        diag -= np.real(np.trace(hdiff))
    omega = (-trace - 0.5 * diag + float(g["omega_clus"])) / 12
    assert abs(omega - float(g["sef"])) < 1e-8, (omega, float(g["sef"]))


@pytest.mark.parametrize("tag", list(LATTICE_CASES))
def test_cpt_and_potthoff_functional(tag):
    g = load_golden(tag)
    lm = _lattice(tag)
    e0, Q, tcs = _cluster(lm)
    z = np.asarray(g["gper_z"])
    K = np.asarray(g["gper_k"], np.float64) @ lm.S.T
    R, els, hdiff, gpos = lm.fourier(False)
    _, tcb, eb = tcs[False]
    e, v = Q[False]
    B, _ = lo.base([(e, v, 1.0)], tcb, eb, hdiff, z)
    G = lo.cpt(B, R, els, K, gpos)
    ref = g["gper"][:, :, 0, 0]
    for iz, zz in enumerate(z):
        tol = 1e-8 if abs(zz.real) < 1e-12 else 1e-6
        assert np.max(np.abs(G[iz] - ref[iz])) < tol, (tag, zz, np.max(np.abs(G[iz] - ref[iz])))
    # Potthoff functional on the 8 (x 8) grid: the lattice part from the
    # oracle, the cluster part the reference's
    w, wt = g["sef_w"], g["sef_wt"]
    grid = (8, 8 if lm.dim >= 2 else 1, 1)
    trace, diag = 0.0, 0.0
    for sd in Q:
        R, els, hdiff, _ = lm.fourier(sd)
        _, tcb, eb = tcs[sd]
        B, ldg = lo.base([(Q[sd][0], Q[sd][1], 1.0)], tcb, eb, hdiff, 1j * w)
        trace += lo.sef_grid(B, ldg, wt, R, els, grid)
        diag -= np.real(np.trace(hdiff))
    if len(Q) == 1:
        trace, diag = 2 * trace, 2 * diag
    omega = (-trace - 0.5 * diag + float(g["omega_clus"])) / len(lm.sites)
    assert abs(omega - float(g["sef"])) < 1e-8, (tag, omega, float(g["sef"]))


def test_cdmft_host_function():
    tag = "lat_cdmft2x2_b4"
    g = load_golden(tag)
    lm = _lattice(tag)
    e0, Q, tcs = _cluster(lm)
    wn = np.array([(2 * n + 1) * np.pi / 50.0 for n in range(20)])
    R, els, hdiff, _ = lm.fourier(False)
    _, tcb, eb = tcs[False]
    e, v = Q[False]
    B, _ = lo.base([(e, v, 1.0)], tcb, eb, hdiff, 1j * wn)
    P = lo.kmean(B, R, els, (8, 8, 1), off=0.5)
    # G_host = P^-1 + Sigma + t_c - z = P^-1 - G^-1 - Gamma (CPT.cpp:356-424)
    G = lo.green(e, v, 1j * wn)
    host = np.linalg.inv(P) - np.linalg.inv(G) - lo.gamma(tcb, eb, 1j * wn)
    assert np.max(np.abs(host - g["host"])) < 1e-8, np.max(np.abs(host - g["host"]))
    # the distance at two bath points against the reference's CDMFT_distance
    # on its own host function
    cm, vals = lm.cluster, lm.cluster_values()
    for key, x in (("dist0", (-1.0, 1.0, 0.5)), ("dist1", (-1.2, 0.8, 0.45))):
        d = lo.cdmft_distance(cm.operators, vals, ["eb1", "eb2", "tb1"], x, cm.n_orb, cm.n_sites,
                              g["host"], wn, np.ones(len(wn)))
        assert abs(d - float(g[key])) < 1e-10 * max(1.0, abs(float(g[key]))), (key, d, g[key])
