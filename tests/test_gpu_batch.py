"""Batched Lanczos ground states (qcmg_lanczos_batch): sectors of different
sizes solved side by side, each from a captured CUDA graph of recurrence
steps, against the host-driven recurrence of qcmg_lanczos_ground_state on
the FP64 path (bit for bit) and against the reference's energies."""
import numpy as np
import pytest

from conftest import load_golden
from models import CASES, hubbard_cluster

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import pyqcm_gb300
    pyqcm_gb300.lib()
    return pyqcm_gb300


def _sectors(pg):
    """Golden sectors (4,900 and 3,920 states), a 3x4 sector (853,776) and
    off-half-filling 3x4 sectors (792 x 924 = 731,808; 495 x 924 = 457,380):
    uneven sizes in one batch."""
    out = []
    for tag in ("chain8", "chain8_n7", "ladder2x4_af", "plaquette_bath4"):
        nx, ny, nb, af, params, sec, _ = CASES[tag]
        ns, nb, ops = hubbard_cluster(nx, ny, nb, af)
        m = pg.ClusterModel(ns, nb)
        for name, (typ, els) in ops.items():
            m.new_operator(name, typ, els)
        out.append((tag, pg.Hamiltonian(m, params, sec)))
    ns, nb, ops = hubbard_cluster(4, 3)
    m = pg.ClusterModel(ns, nb)
    for name, (typ, els) in ops.items():
        m.new_operator(name, typ, els)
    params = {"t": 1.0, "tp": -0.3, "U": 8.0, "mu": 4.0}
    for sec in ("R0:N12:S0", "R0:N11:S1", "R0:N10:S2"):
        out.append((sec, pg.Hamiltonian(m, params, sec)))
    return out


def test_batch_matches_single_sector_lanczos_bitwise(pg):
    secs = _sectors(pg)
    hs = [h for _, h in secs]
    res = pg.lanczos_batch(hs, want_psi=True, tol=1e-12, max_iter=1000, chunk=16)
    for (tag, h), (e0, psi, nit) in zip(secs, res):
        h.set_path(False)
        e1, psi1, alpha1, _ = h.lanczos(tol=1e-12, max_iter=1000)
        assert e0 == e1, (tag, e0, e1)
        assert nit == len(alpha1), (tag, nit, len(alpha1))
        assert np.array_equal(psi, psi1), tag
    for tag in ("chain8", "chain8_n7", "ladder2x4_af", "plaquette_bath4"):
        g = load_golden(tag)
        e0 = res[[t for t, _ in secs].index(tag)][0]
        assert abs(e0 - float(g["lz_E0"])) <= 1e-10 * abs(float(g["lz_E0"])), tag


def test_batch_chunk_size_does_not_change_the_result(pg):
    secs = _sectors(pg)[:4]
    hs = [h for _, h in secs]
    a = pg.lanczos_batch(hs, tol=1e-12, chunk=2)
    b = pg.lanczos_batch(hs, tol=1e-12, chunk=64)
    for (ea, _, na), (eb, _, nb) in zip(a, b):
        assert ea == eb and na == nb


def test_batch_reports_no_convergence(pg):
    secs = _sectors(pg)[:2]
    with pytest.raises(pg.QcmgError):
        pg.lanczos_batch([h for _, h in secs], tol=1e-12, max_iter=5, chunk=4)


def test_batch_over_every_sector_of_an_impurity(pg):
    """Every (N_up >= N_dn) sector of the 2x2 plaquette with 4 bath orbitals
    (45 sectors of 1 to 4,900 states, the empty and the full one included)
    in one batch: bit-for-bit the single-sector recurrence, and on the
    sectors of at most 200 states the lowest eigenvalue of the dense matrix
    built column by column from the product (1e-10)."""
    from pyqcm_gb300.cdmft import plaquette_bath_model
    lm = plaquette_bath_model(4, "R0:N8:S0")
    lm.finalize()
    vals = {"t": 1.0, "U": 4.0, "mu": 1.7, "eb1": -1.0, "eb2": 1.1, "eb3": -0.6, "eb4": 0.7,
            "tb1": 0.5, "tb2": 0.45, "tb3": 0.4, "tb4": 0.35}
    no = 8
    secs = [f"R0:N{u + d}:S{u - d}" for u in range(no + 1) for d in range(u + 1)]
    hs = [pg.Hamiltonian(lm.cluster, vals, s) for s in secs]
    for h in hs:
        h.set_path(False)
    assert min(h.dim for h in hs) == 1 and max(h.dim for h in hs) == 4900
    res = pg.lanczos_batch(hs, tol=1e-12, max_iter=1000, chunk=16)
    for s, h, (e0, _, nit) in zip(secs, hs, res):
        e1, _, alpha1, _ = h.lanczos(tol=1e-12, max_iter=1000, want_psi=False)
        assert e0 == e1 and nit == len(alpha1), (s, e0, e1, nit, len(alpha1))
        if h.dim <= 200:
            D = np.zeros((h.dim, h.dim))
            for i in range(h.dim):
                e = np.zeros(h.dim)
                e[i] = 1.0
                D[:, i] = h.matvec(e)
            assert abs(np.linalg.eigvalsh(0.5 * (D + D.T))[0] - e0) < 1e-10, s
