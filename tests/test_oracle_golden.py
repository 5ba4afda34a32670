"""The CPU oracle (oracle/) against the reference's own outputs
(tests/golden, generated by tests/golden/make_golden.py from the reference's
C++ compiled in oracle/refbuild).  No GPU needed."""
import numpy as np
import pytest

import qcm_oracle as qo
from conftest import load_golden
from helpers import case_model, csr_dense, halfop_dense_from_ref, oracle_sector
from models import CASES, ZS


def test_halfbasis_bit_exact():
    g = load_golden("halfbasis")
    for key, ref in g.items():
        if not key.startswith("halfbasis_"):
            continue
        _, L, N = key.split("_")
        got = qo.halfbasis(int(L[1:]), int(N[1:]))
        assert got.dtype == np.uint32
        assert np.array_equal(got, ref), key


def test_rank_matches_binary_search():
    bs = qo.halfbasis(12, 6)
    lib = qo.lib()
    for i in (0, 1, 100, 923):
        assert lib.qo_rank(bs.ctypes.data_as(qo.ctypes.POINTER(qo.ctypes.c_uint32)), len(bs),
                           int(bs[i])) == i


@pytest.mark.parametrize("tag", list(CASES))
def test_halfop_tables_match_reference(tag):
    g = load_golden(tag)
    S, (up, dn, pr) = oracle_sector(tag)
    ns, nb, ops, params, sec = case_model(tag)
    names = [k for k in ops if ops[k][0] == "one-body" and k in params]
    for spin, T_or, dim in ((0, S.up, S.du), (1, S.dn, S.dd)):
        sfx = "dn" if spin else "up"
        T_ref = halfop_dense_from_ref(g, "h", [f"{n}_{sfx}" for n in names], params, dim)
        assert np.allclose(csr_dense(*T_or), T_ref, atol=1e-14, rtol=0), (tag, spin)


@pytest.mark.parametrize("tag", list(CASES))
def test_matvec_and_start_vector(tag):
    g = load_golden(tag)
    S, _ = oracle_sector(tag)
    x0 = qo.seeded_start(S.dim, 0)
    assert np.max(np.abs(x0 - g["h_x0"])) < 1e-15
    y = S.matvec(g["h_x0"])
    assert np.max(np.abs(y - g["h_Hx0"])) <= 1e-13 * np.max(np.abs(g["h_Hx0"]))
    y4 = S.matvec(g["h_x0"], nthreads=4)
    assert np.max(np.abs(y4 - y)) == 0.0


@pytest.mark.parametrize("tag", list(CASES))
def test_lanczos_energy_and_vector(tag):
    g = load_golden(tag)
    S, _ = oracle_sector(tag)
    x0 = g["h_x0"]
    al, be, e0 = qo.lanczos_eigenvalue(S.mult_add, x0)
    assert abs(e0 - g["lz_E0"]) <= 1e-10 * abs(g["lz_E0"])
    assert abs(len(al) - len(g["lz_alpha"])) <= 2
    psi = qo.lanczos_eigenvector(S.mult_add, x0, al, be)
    ov = abs(psi @ g["lz_psi"]) / (np.linalg.norm(psi) * np.linalg.norm(g["lz_psi"]))
    assert ov > 1 - 1e-10
    assert abs(g["gs_E0"] - g["lz_E0"]) < 1e-10 * abs(g["gs_E0"])


def test_create_destroy_bit_exact():
    g = load_golden("chain8")
    for tag, orb, pm in (("dup", 3, -1), ("ddn", 5 + 8, -1), ("cup", 2, 1), ("cdn", 6 + 8, 1)):
        y = qo.apply_c(8, orb, pm, 4, 4, g[tag + "_x"])
        assert np.array_equal(y, g[tag + "_y"]), tag


@pytest.mark.parametrize("tag", [t for t in CASES if CASES[t][6]])
def test_green_function_from_oracle_qmatrix(tag):
    g = load_golden(tag)
    ns, nb, ops, params, sec = case_model(tag)
    S, (up, dn, pr) = oracle_sector(tag)
    L = ns + nb
    al, be, e0 = qo.lanczos_eigenvalue(S.mult_add, g["h_x0"])
    psi = qo.lanczos_eigenvector(S.mult_add, g["h_x0"], al, be)

    def mao(nu, nd):
        s = qo.Sector(L, nu, nd, up, dn, pr)
        return s.mult_add, s.dim

    af = CASES[tag][3]
    for spin_down in ((False, True) if af else (False,)):
        e, v = qo.qmatrix_for_state(mao, L, S.nup, S.ndn, psi, e0, range(ns), spin_down)
        q = "qdn" if spin_down else "qup"
        assert_qmatrix_parity(e, v, g[q + "_e"], g[q + "_v"].T)
        for k, z in enumerate(ZS):
            G = qo.green_function(e, v, z)
            ref = g[("gzdn" if spin_down else "gz") + str(k)]
            assert np.max(np.abs(G - ref)) < 1e-8, (tag, spin_down, k)


def assert_qmatrix_parity(e, v, e_ref, v_ref, elow=2.0, wmin=1e-4, tol=1e-8):
    """Parity of two Q-matrices computed by band Lanczos.  Band Lanczos
    converges the low-energy poles first and stops on the lowest eigenvalue
    of the projected matrix (Lanczos.hpp:340-375), so poles far from the Fermi
    level are not converged in either run and move by ~1e-5 under rounding
    changes.  Parity is therefore checked where the method converges:
      - the sum rule Q Q^dagger = 1 (Q_matrix::check_norm) to 1e-8 (streamline
        drops poles of weight < Qmatrix_vtol = 1e-10, Q_matrix.hpp:191-205);
      - every pole with |e| < elow and weight > wmin matches to tol;
      - G(i w_n) on a Matsubara grid (beta = 50) matches to tol."""
    L = v.shape[0]
    assert np.max(np.abs(v @ v.conj().T - np.eye(L))) < 1e-8
    w = np.sum(np.abs(v) ** 2, axis=0)
    for ei, wi in zip(e, w):
        if abs(ei) < elow and wi > wmin:
            assert np.min(np.abs(e_ref - ei)) < tol, (ei, wi)
    for n in range(0, 400, 7):
        z = 1j * (2 * n + 1) * np.pi / 50.0
        G = qo.green_function(e, v, z)
        Gr = qo.green_function(e_ref, v_ref, z)
        assert np.max(np.abs(G - Gr)) < tol, z


@pytest.mark.parametrize("tag", ["chain8", "ladder2x4_af", "plaquette_bath4"])
def test_continued_fraction_green_function_against_reference(tag):
    """The oracle's restatement of the continued-fraction Green function
    (GF_method 'F': LanczosGreen per orbital pair, Lanczos.hpp:156-183, and
    continued_fraction_set::Green_function) against the reference's own G(z)
    from its build_cf."""
    g = load_golden(tag)
    gcf = load_golden(tag + "_cf")
    ns, nb, ops, params, sec = case_model(tag)
    S, (up, dn, pr) = oracle_sector(tag)
    L = ns + nb
    al, be, e0 = qo.lanczos_eigenvalue(S.mult_add, g["h_x0"])
    assert abs(e0 - gcf["gs_E0"]) < 1e-10 * abs(e0)
    psi = qo.lanczos_eigenvector(S.mult_add, g["h_x0"], al, be)

    def mao(nu, nd):
        s = qo.Sector(L, nu, nd, up, dn, pr)
        return s.mult_add, s.dim

    af = CASES[tag][3]
    for spin_down in ((False, True) if af else (False,)):
        G = qo.cf_green_function_for_state(mao, L, S.nup, S.ndn, psi, e0, 1.0, list(range(ns)),
                                           ZS, spin_down)
        for k in range(len(ZS)):
            ref = gcf[("gzdn" if spin_down else "gz") + str(k)]
            assert np.max(np.abs(G[k] - ref)) < 1e-9, (tag, spin_down, k, np.max(np.abs(G[k] - ref)))


@pytest.mark.parametrize("tag", ["chain8", "ladder2x4_af", "plaquette_bath4"])
def test_matrix_continued_fraction_green_function_against_reference(tag):
    """The oracle's restatement of the matrix continued fraction (GF_method
    'M': start-block factor, blockLanczosSVD, matrix_continued_fraction,
    mcf_set) against the reference's own G(z) from its build_mcf."""
    g = load_golden(tag)
    gm = load_golden(tag + "_mcf")
    ns, nb, ops, params, sec = case_model(tag)
    S, (up, dn, pr) = oracle_sector(tag)
    L = ns + nb
    al, be, e0 = qo.lanczos_eigenvalue(S.mult_add, g["h_x0"])
    assert abs(e0 - gm["gs_E0"]) < 1e-10 * abs(e0)
    psi = qo.lanczos_eigenvector(S.mult_add, g["h_x0"], al, be)

    def mao(nu, nd):
        s = qo.Sector(L, nu, nd, up, dn, pr)
        return s.mult_add, s.dim

    af = CASES[tag][3]
    for spin_down in ((False, True) if af else (False,)):
        G = qo.mcf_green_function_for_state(mao, L, S.nup, S.ndn, psi, e0, 1.0, list(range(ns)),
                                            ZS, spin_down)
        for k in range(len(ZS)):
            ref = gm[("gzdn" if spin_down else "gz") + str(k)]
            assert np.max(np.abs(G[k] - ref)) < 1e-10, (tag, spin_down, k, np.max(np.abs(G[k] - ref)))


def test_band_lanczos_vector_kernels():
    """The oracle's batched vector kernels against numpy, and the dot
    products equal on 1 and 4 threads (fixed-chunk sums)."""
    rng = np.random.default_rng(3)
    n = 100_003
    vs = [rng.standard_normal(n) for _ in range(5)]
    w = rng.standard_normal(n)
    d1 = qo._multidot(vs, w, 1)
    d4 = qo._multidot(vs, w, 4)
    assert np.array_equal(d1, d4)
    assert np.allclose(d1, [v @ w for v in vs], rtol=1e-13, atol=1e-10)
    coef = rng.standard_normal(5)
    ref = [v - c * w for v, c in zip(vs, coef)]
    got = [v.copy() for v in vs]
    qo._sub_rank1(got, coef, w, 4)
    assert all(np.max(np.abs(a - b)) < 1e-12 for a, b in zip(got, ref))  # FMA or not
    y = w.copy()
    qo._sub_combination(vs, coef, y, 4)
    ref_y = w.copy()
    for v, c in zip(vs, coef):
        ref_y = ref_y - c * v
    assert np.max(np.abs(y - ref_y)) < 1e-12
