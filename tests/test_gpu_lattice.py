"""GPU parity of the lattice integrals (CPT periodized G, Potthoff
functional on a fixed grid, density of states, CDMFT host and distance) against the
reference's QCM layer (tests/golden/lat_*.npz)."""
import numpy as np
import pytest

from conftest import load_golden
from lattice_helpers import build_lattice
from models import LATTICE_CASES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import pyqcm_gb300
    pyqcm_gb300.lib()
    return pyqcm_gb300


@pytest.mark.parametrize("tag", list(LATTICE_CASES))
def test_cpt_periodized_green_function(pg, tag):
    g = load_golden(tag)
    inst = build_lattice(tag).instance()
    G = inst.periodized_Green_function(g["gper_z"], g["gper_k"])
    ref = g["gper"][:, :, 0, 0]
    for iz, z in enumerate(g["gper_z"]):
        tol = 1e-8 if abs(z.real) < 1e-12 else 1e-6  # real axis: band-Lanczos poles (see Q-matrix parity)
        assert np.max(np.abs(G[iz] - ref[iz])) < tol, (tag, z)


@pytest.mark.parametrize("tag", list(LATTICE_CASES))
def test_potthoff_functional_grid(pg, tag):
    from pyqcm_gb300 import lattice as lat
    g = load_golden(tag)
    lm = build_lattice(tag)
    inst = lm.instance()
    assert abs(inst.cluster.Potthoff_functional() - g["omega_clus"]) < 1e-9
    lat.set_wavevector_grid(8, 8 if lm.dim >= 2 else 1, 1)
    lat.discrete_integration_grid(g["sef_w"], g["sef_wt"])
    om = inst.Potthoff_functional()
    assert abs(om - g["sef"]) < 1e-8, (om, float(g["sef"]))


@pytest.mark.parametrize("tag", list(LATTICE_CASES))
def test_density_of_states_grid(pg, tag):
    """DoS on the 8 (x 8) wavevector grid at six frequencies w + 0.1 i
    against the reference's QCM::dos (use_grid): both spin columns.  The
    real-axis tolerance is the CPT one (band-Lanczos poles far from the Fermi
    level, see the Q-matrix parity note)."""
    from pyqcm_gb300 import lattice as lat
    g = load_golden(tag)
    lm = build_lattice(tag)
    inst = lm.instance()
    lat.set_wavevector_grid(8, 8 if lm.dim >= 2 else 1, 1)
    D = inst.dos(g["dos_z"])
    assert D.shape == g["dos"].shape
    assert np.max(np.abs(D - g["dos"])) < 1e-6, (tag, np.max(np.abs(D - g["dos"])))


def test_cdmft_host_and_distance(pg):
    tag = "lat_cdmft2x2_b4"
    g = load_golden(tag)
    inst = build_lattice(tag).instance()
    wn = np.array([(2 * n + 1) * np.pi / 50.0 for n in range(20)])
    host = inst.CDMFT_host(wn, np.ones(len(wn)), kside=8)[False]
    assert np.max(np.abs(host - g["host"])) < 1e-8
    d0 = inst.CDMFT_distance({"eb1_1": -1.0, "eb2_1": 1.0, "tb1_1": 0.5})
    d1 = inst.CDMFT_distance({"eb1_1": -1.2, "eb2_1": 0.8, "tb1_1": 0.45})
    assert abs(d0 - g["dist0"]) < 1e-10 * max(1.0, abs(float(g["dist0"])))
    assert abs(d1 - g["dist1"]) < 1e-10 * max(1.0, abs(float(g["dist1"])))


@pytest.mark.parametrize("tag", list(LATTICE_CASES))
def test_lattice_averages_grid(pg, tag):
    """Averages of the one-body operators (t, the density wave, mu) on the
    Potthoff-functional grids against the reference's QCM::averages (grid
    frequencies, wavevector grid)."""
    from pyqcm_gb300 import lattice as lat
    g = load_golden(tag)
    lm = build_lattice(tag)
    inst = lm.instance()
    lat.set_wavevector_grid(8, 8 if lm.dim >= 2 else 1, 1)
    lat.discrete_integration_grid(g["sef_w"], g["sef_wt"])
    names = [str(n) for n in g["ave_ops"]]
    ave = inst.averages(names)
    assert list(ave) == names
    got = np.array([ave[n] for n in names])
    assert np.max(np.abs(got - g["ave"])) < 1e-9, (tag, got, g["ave"])


@pytest.mark.parametrize("tag", list(LATTICE_CASES))
def test_potential_energy_grid(pg, tag):
    """Potential energy per site on the Potthoff-functional grids against the
    reference's QCM::potential_energy (grid frequencies, wavevector grid),
    including its extrapolated Tr Sigma(infinity)."""
    from pyqcm_gb300 import lattice as lat
    g = load_golden(tag)
    lm = build_lattice(tag)
    inst = lm.instance()
    lat.set_wavevector_grid(8, 8 if lm.dim >= 2 else 1, 1)
    lat.discrete_integration_grid(g["sef_w"], g["sef_wt"])
    e = inst.potential_energy()
    assert abs(e - g["epot"]) < 1e-8, (tag, e, float(g["epot"]))


def test_lattice_stage_from_a_qmatrix_file(pg, tmp_path):
    """The impurity stage written to a Q-matrix file and read back by a fresh
    instance gives the same Potthoff functional and CPT Green function, with
    no impurity solve in the second instance."""
    from pyqcm_gb300 import lattice as lat
    g = load_golden("lat_vca2x2_af")
    lat.set_wavevector_grid(8, 8, 1)
    lat.discrete_integration_grid(g["sef_w"], g["sef_wt"])
    a = build_lattice("lat_vca2x2_af").instance()
    om_a = a.Potthoff_functional()
    G_a = a.periodized_Green_function(g["gper_z"], g["gper_k"])
    path = tmp_path / "vca.npz"
    a.cluster.write_qmatrix(path)
    b = build_lattice("lat_vca2x2_af").instance()
    b.cluster.read_qmatrix(path)
    assert not b.cluster._H  # no sector Hamiltonian was built
    assert b.Potthoff_functional() == om_a
    assert np.array_equal(b.periodized_Green_function(g["gper_z"], g["gper_k"]), G_a)
