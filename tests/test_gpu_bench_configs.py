"""GPU parity on the benchmarked configurations against the reference's own
code (goldens written by tests/golden/make_golden.py from oracle/_ref):

- the 4x4 Hubbard cluster at half filling (165,636,900 states) and the 3x4
  cluster with diagonal hopping (853,776 states): one product y = H x0 on
  the reference's seeded start vector (sum, sum of squares, <x0, y> and 4096
  sampled elements) and the Lanczos ground-state energy at
  accur_lanczos = 1e-10, on both arithmetic paths;
- the 2x2 plaquette + 8 bath orbitals (8 energies, 16 hybridizations) of the
  batched-CDMFT configuration: ground-state energy, cluster Green function at
  Matsubara frequencies, the CDMFT host function on the 64x64 k grid at the
  200 Matsubara frequencies of beta = 50, and CDMFT distances;
- the 3x4 VCA case (Neel Weiss field M_1 = 0.1): ground-state energy, the
  converged poles of both spin blocks, and the Potthoff functional on the
  128x128 k grid x 256 Gauss-Legendre frequencies.
"""
import os

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def pg():
    import pyqcm_gb300
    pyqcm_gb300.lib()
    return pyqcm_gb300


def _golden_or_skip(tag):
    if not os.path.exists(os.path.join(HERE, "golden", tag + ".npz")):
        pytest.skip(f"golden {tag} not generated")
    return load_golden(tag)


def _hamiltonian(pg, nx, ny, params, sector):
    from models import hubbard_cluster
    ns, nb, ops = hubbard_cluster(nx, ny)
    m = pg.ClusterModel(ns, nb)
    for name, (typ, els) in ops.items():
        m.new_operator(name, typ, els)
    return pg.Hamiltonian(m, params, sector)


LARGE = {
    "large_4x4": (4, 4, {"t": 1.0, "U": 8.0, "mu": 4.0}, "R0:N16:S0"),
    "large_3x4": (3, 4, {"t": 1.0, "tp": -0.3, "U": 8.0, "mu": 4.0}, "R0:N12:S0"),
}


@pytest.fixture(scope="module")
def seeded_x0():
    cache = {}

    def get(dim):
        if dim not in cache:
            import qcm_oracle as qo
            cache.clear()
            cache[dim] = qo.seeded_start(dim, 0)
        return cache[dim]
    return get


@pytest.mark.parametrize("tag", list(LARGE))
@pytest.mark.parametrize("path", ["fixed_point", "fp64"])
def test_large_sector_product_checksum(pg, seeded_x0, tag, path):
    """y = H x0 on the reference's seeded start vector, against its serial
    Hamiltonian_Factorized::mult_add: 4096 sampled elements to 1e-13 of
    max|y|, and the sum, sum of squares and <x0, y> to 1e-11 relative."""
    g = _golden_or_skip(tag)
    nx, ny, params, sec = LARGE[tag]
    H = _hamiltonian(pg, nx, ny, params, sec)
    assert H.dim == int(g["h_dim"])
    if path == "fixed_point" and not H.fx_available():
        pytest.skip("the fixed-point path does not apply to this Hamiltonian")
    H.set_path(path == "fixed_point")
    x0 = seeded_x0(H.dim)
    y = H.matvec(x0)
    at = g["h_at"].astype(np.int64)
    ymax = float(np.max(np.abs(y)))
    assert np.max(np.abs(y[at] - g["h_y"])) <= 1e-13 * ymax
    for key, val in (("h_sum", np.sum(y)), ("h_norm2", np.dot(y, y)), ("h_xy", np.dot(x0, y))):
        ref = float(g[key])
        assert abs(val - ref) <= 1e-11 * max(1.0, abs(ref)), (key, val, ref)


@pytest.mark.parametrize("tag", list(LARGE))
@pytest.mark.parametrize("path", ["fixed_point", "fp64"])
def test_large_sector_lanczos_energy(pg, tag, path):
    """Lanczos ground-state energy from the reference's seeded start at
    accur_lanczos = 1e-10, against its LanczosEigenvalue: 1e-10 relative."""
    g = _golden_or_skip(tag)
    nx, ny, params, sec = LARGE[tag]
    H = _hamiltonian(pg, nx, ny, params, sec)
    if path == "fixed_point" and not H.fx_available():
        pytest.skip("the fixed-point path does not apply to this Hamiltonian")
    H.set_path(path == "fixed_point")
    e0, _, alpha, _ = H.lanczos(tol=1e-10, max_iter=1000, want_psi=False)
    ref = float(g["lz_E0"])
    assert abs(e0 - ref) <= 1e-10 * abs(ref), (e0, ref)
    # the first recurrence coefficients follow the reference's own
    n = min(len(alpha), len(g["lz_alpha"]), 20)
    assert np.max(np.abs(alpha[:n] - g["lz_alpha"][:n])) < 1e-9


def test_large_4x4_reorthogonalized_lanczos(pg):
    """Full reorthogonalization on the 4x4 half-filled sector with at most
    150 vectors held in HBM (restarting from the Ritz vector at the cap):
    the energy matches the reference's LanczosEigenvalue to 1e-10."""
    g = _golden_or_skip("large_4x4")
    nx, ny, params, sec = LARGE["large_4x4"]
    H = _hamiltonian(pg, nx, ny, params, sec)
    e0, _, _, _ = H.lanczos(tol=1e-10, max_iter=1000, reorth=150, want_psi=False)
    ref = float(g["lz_E0"])
    assert abs(e0 - ref) <= 1e-10 * abs(ref), (e0, ref)
    st = H.lanczos_stats()
    assert st["vectors"] <= 150 and st["reorth_ms"] > 0.0


def test_cdmft_plaquette_8bath(pg):
    """Batched-CDMFT model at one parameter point against the reference's ED
    and QCM layers (64x64 k grid, 200 Matsubara frequencies)."""
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import BENCH_C4_PARAMS
    from pyqcm_gb300.cdmft import bath_names, plaquette_bath_model
    g = _golden_or_skip("bench_cdmft2x2_b8")
    lm = plaquette_bath_model(8, "R0:N12:S0", hybridizations=2)
    lm.set_parameters(dict(BENCH_C4_PARAMS))
    inst = lm.instance()
    E0, _ = inst.ground_state()
    assert abs(E0 - float(g["gs_E0"])) <= 1e-10 * abs(float(g["gs_E0"]))
    wn = g["host_w"]
    for k, n in enumerate(g["gz_n"]):
        G = inst.cluster.Green_function(1j * wn[n])
        assert np.max(np.abs(G[:4, :4] - g[f"gz{k}"][:4, :4])) < 1e-8, n
    host = inst.CDMFT_host(wn, np.ones(len(wn)), kside=64)[False]
    assert np.max(np.abs(host - g["host"])) < 1e-8
    names = bath_names(8, 2)
    for key, p in (("dist0", g["dist_p0"]), ("dist1", g["dist_p1"])):
        d = inst.CDMFT_distance(dict(zip(names, p)))
        ref = float(g[key])
        assert abs(d - ref) < 1e-10 * max(1.0, abs(ref)), (key, d, ref)


def _vca_3x4(pg):
    from pyqcm_gb300.lattice import LatticeModel
    cm = pg.ClusterModel(12, 0)
    sites = [(x, y, 0) for y in range(3) for x in range(4)]
    lm = LatticeModel(cm, sites, [(4, 0, 0), (1, 3, 0)])
    lm.interaction_operator("U", 1.0)
    lm.hopping_operator("t", (1, 0, 0), -1.0)
    lm.hopping_operator("t", (0, 1, 0), -1.0)
    lm.hopping_operator("tp", (1, 1, 0), -1.0)
    lm.hopping_operator("tp", (-1, 1, 0), -1.0)
    lm.density_wave("M", "Z", (1, 1, 0), 1.0, 0.0)
    lm.set_target_sectors("R0:N12:S0")
    lm.set_parameters({"t": 1.0, "tp": -0.3, "U": 8.0, "mu": 4.0, "M": 0.0, "M_1": 0.1})
    return lm


def test_vca_3x4_potthoff_functional(pg):
    """3x4 VCA case: E0, the converged poles of both spin blocks (|e| < 2,
    weight > 1e-4), the cluster part of Omega, and the Potthoff functional on
    the full 128x128 x 256 grid, against the reference."""
    from pyqcm_gb300 import lattice as lat
    from test_oracle_golden import assert_qmatrix_parity
    g = _golden_or_skip("bench_vca3x4")
    lm = _vca_3x4(pg)
    inst = lm.instance()
    E0, _ = inst.ground_state()
    assert abs(E0 - float(g["gs_E0"])) <= 1e-10 * abs(float(g["gs_E0"]))
    for spin_down, key in ((False, "qup"), (True, "qdn")):
        e, v = inst.cluster.qmatrix(spin_down)
        assert_qmatrix_parity(e, v, g[key + "_e"], g[key + "_v"].T)
    assert abs(inst.cluster.Potthoff_functional() - float(g["omega_clus"])) < 1e-9
    lat.set_wavevector_grid(128, 128, 1)
    lat.discrete_integration_grid(g["sef_w"], g["sef_wt"])
    om = inst.Potthoff_functional()
    assert abs(om - float(g["sef"])) < 1e-8, (om, float(g["sef"]))
    # the same number bit for bit whatever block size the point kernel runs
    # with (the per-frequency sums are taken in a fixed order)
    import os
    got = []
    for T in ("32", "64", "96"):
        os.environ["QCMG_POINT_THREADS"] = T
        try:
            got.append(inst.Potthoff_functional())
        finally:
            del os.environ["QCMG_POINT_THREADS"]
    assert got == [om, om, om], (got, om)
