"""GPU parity of the exact-diagonalization path: the engine (libqcmg through
its C ABI) against the reference's own outputs (tests/golden) and the CPU
oracle on the same seeded inputs."""
import math

import numpy as np
import pytest

import qcm_oracle as qo
from conftest import load_golden
from helpers import case_model, csr_dense, engine_model, halfop_dense_from_ref, oracle_sector
from models import CASES, ZS
from test_oracle_golden import assert_qmatrix_parity

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import pyqcm_gb300
    pyqcm_gb300.lib()
    return pyqcm_gb300


def test_halfbasis_bit_exact(pg):
    g = load_golden("halfbasis")
    for key, ref in g.items():
        if key.startswith("halfbasis_"):
            _, L, N = key.split("_")
            got = pg.halfbasis(int(L[1:]), int(N[1:]))
            assert np.array_equal(got, ref), key
    # larger and edge cases against the oracle
    for L, N in ((16, 8), (20, 10), (24, 3), (5, 0), (5, 5), (1, 1)):
        assert np.array_equal(pg.halfbasis(L, N), qo.halfbasis(L, N)), (L, N)


def test_halfbasis_rank(pg):
    bs = qo.halfbasis(16, 8)
    assert np.array_equal(pg.halfbasis_rank(16, 8, bs), np.arange(len(bs), dtype=np.uint32))
    # states outside the basis rank to dim
    bad = np.array([0, 0xffff, 1 << 17, 0b111], np.uint32)
    assert np.all(pg.halfbasis_rank(16, 8, bad) == len(bs))


@pytest.mark.parametrize("tag", list(CASES))
def test_halfop_tables_match_reference(pg, tag):
    g = load_golden(tag)
    m, params, sec = engine_model(tag)
    H = pg.Hamiltonian(m, params, sec)
    ns, nb, ops, _, _ = case_model(tag)
    names = [k for k in ops if ops[k][0] == "one-body" and k in params]
    for spin, dim in ((0, H.dim_up), (1, H.dim_dn)):
        sfx = "dn" if spin else "up"
        T_ref = halfop_dense_from_ref(g, "h", [f"{n}_{sfx}" for n in names], params, dim)
        T_gpu = csr_dense(*H.halfop(spin))
        # index pattern bit-exact, values exact sums of the same doubles
        assert np.array_equal(T_gpu != 0, T_ref != 0), (tag, spin)
        assert np.allclose(T_gpu, T_ref, atol=1e-14, rtol=0), (tag, spin)


@pytest.mark.parametrize("tag", list(CASES))
def test_matvec_matches_reference(pg, tag):
    g = load_golden(tag)
    m, params, sec = engine_model(tag)
    H = pg.Hamiltonian(m, params, sec)
    x = g["h_x0"]
    y = H.matvec(x)
    ref = g["h_Hx0"]
    assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref))
    # accumulate form: y += H x
    y2 = np.ones(H.dim)
    H.mult_add(x, y2)
    assert np.max(np.abs(y2 - 1.0 - ref)) <= 1e-13 * np.max(np.abs(ref))


# The fixed-point path applies to one hop magnitude per spin: of the golden
# cases, the chains (the ladder has t and t', the plaquette bath
# hybridizations); the others are tested on the FP64 path only.
LANCZOS_IDS = [("fixed_point", t) for t in ("chain8", "chain8_n7")] + [("fp64", t) for t in CASES]


@pytest.mark.parametrize("path,tag", LANCZOS_IDS)
def test_lanczos_ground_state(pg, tag, path):
    g = load_golden(tag)
    m, params, sec = engine_model(tag)
    H = pg.Hamiltonian(m, params, sec)
    if path == "fixed_point":
        assert H.fx_available()  # the id really runs the fixed-point path
    H.set_path(path == "fixed_point")
    e0, psi, al, be = H.lanczos()  # seeded start, as the reference's states()
    assert abs(e0 - g["lz_E0"]) <= 1e-10 * abs(g["lz_E0"])
    assert abs(len(al) - len(g["lz_alpha"])) <= 2
    ov = abs(psi @ g["lz_psi"]) / (np.linalg.norm(psi) * np.linalg.norm(g["lz_psi"]))
    assert ov > 1 - 1e-10
    # first recurrence coefficients agree closely (before rounding drift)
    assert np.max(np.abs(al[:10] - g["lz_alpha"][:10])) < 1e-10


@pytest.mark.parametrize("tag", ["chain8", "ladder2x4_af"])
def test_lanczos_reorth(pg, tag):
    g = load_golden(tag)
    m, params, sec = engine_model(tag)
    H = pg.Hamiltonian(m, params, sec)
    e0, psi, al, be = H.lanczos(reorth=200)
    assert abs(e0 - g["lz_E0"]) <= 1e-10 * abs(g["lz_E0"])
    r = H.matvec(psi) - e0 * psi
    assert np.linalg.norm(r) < 1e-8


def test_create_destroy_bit_exact(pg):
    g = load_golden("chain8")
    for tag, orb, pm in (("dup", 3, -1), ("ddn", 5 + 8, -1), ("cup", 2, 1), ("cdn", 6 + 8, 1)):
        y = pg.apply_c(8, orb, pm, 4, 4, g[tag + "_x"])
        assert np.array_equal(y, g[tag + "_y"]), tag


def test_device_start_vectors_match_host_path(pg):
    """c / c^dagger applied on the device with the start vectors left there
    (apply_c_device + build_Q_matrix_device) gives bit for bit the host
    path's vectors and Q-matrix (apply_c + build_Q_matrix)."""
    torch = _torch()
    m, params, sec = engine_model("chain8")
    inst = pg.ModelInstance(m, params, sec)
    inst.ground_state()
    st = inst.states[0]
    L, ns = m.n_orb, m.n_sites
    for pm in (-1, 1):
        H = inst.hamiltonian(st.sec.nup + pm, st.sec.ndn)
        phi = [pg.apply_c(L, o, pm, st.sec.nup, st.sec.ndn, st.psi) for o in range(ns)]
        phi_d = pg.ed.apply_c_device(L, list(range(ns)), pm, st.sec.nup, st.sec.ndn,
                                     torch.from_numpy(st.psi).cuda())
        assert np.array_equal(phi_d.cpu().numpy(), np.array(phi))
        e_h, Q_h = H.build_Q_matrix(phi)
        e_d, Q_d = H.build_Q_matrix_device(phi_d)
        assert np.array_equal(e_h, e_d) and np.array_equal(Q_h, Q_d), pm


@pytest.mark.parametrize("tag", [t for t in CASES if CASES[t][6]])
def test_green_function_pipeline(pg, tag):
    """ground state -> c/c^dagger -> band Lanczos -> Q-matrix -> G(z), all on
    the GPU, against the reference's Q-matrix and G(z)."""
    g = load_golden(tag)
    m, params, sec = engine_model(tag)
    inst = pg.ModelInstance(m, params, sec)
    E0, gs_sec = inst.ground_state()
    assert abs(E0 - g["gs_E0"]) <= 1e-10 * abs(g["gs_E0"])
    af = CASES[tag][3]
    for spin_down in ((False, True) if af else (False,)):
        e, v = inst.qmatrix(spin_down)
        q = "qdn" if spin_down else "qup"
        assert_qmatrix_parity(e, v, g[q + "_e"], g[q + "_v"].T)
        for k, z in enumerate(ZS):
            G = inst.Green_function(z, spin_down)
            ref = g[("gzdn" if spin_down else "gz") + str(k)]
            assert np.max(np.abs(G - ref)) < 1e-8, (tag, spin_down, k)
    assert abs(inst.Potthoff_functional() - g["omega"]) < 1e-8
    if CASES[tag][2]:
        for k, z in enumerate(ZS):
            assert np.max(np.abs(inst.hybridization_function(z) - g[f"hyb{k}"])) < 1e-12
            # Sigma carries G^-1: G's 1e-8 tolerance propagates as
            # 1e-8 |G^-1|^2 (the same bound for the device path)
            Gi = np.linalg.inv(g[f"gz{k}"])
            tol = 1e-8 * max(1.0, np.linalg.norm(Gi, 2) ** 2)
            assert np.max(np.abs(inst.self_energy(z) - g[f"sig{k}"])) < tol
            S, Gm = inst.self_energy_device([z], want_gamma=True)
            assert np.max(np.abs(S[0] - g[f"sig{k}"])) < tol
            assert np.max(np.abs(Gm[0] - g[f"hyb{k}"])) < 1e-12


@pytest.mark.parametrize("method", ["F", "M"])
@pytest.mark.parametrize("tag", ["chain8", "ladder2x4_af", "plaquette_bath4"])
def test_continued_fraction_green_function(pg, tag, method):
    """GF_method 'F': ground state -> c/c^dagger per orbital pair ->
    continued-fraction Lanczos on the GPU -> G(z); GF_method 'M': the start
    block of all orbitals -> block Lanczos on the GPU -> matrix continued
    fraction.  Both against the reference's own G(z) from build_cf /
    build_mcf."""
    g = load_golden(tag + ("_cf" if method == "F" else "_mcf"))
    m, params, sec = engine_model(tag)
    pg.set_global_parameter("GF_method", method)
    try:
        inst = pg.ModelInstance(m, params, sec)
    finally:
        pg.set_global_parameter("GF_method", "L")
    E0, _ = inst.ground_state()
    assert abs(E0 - g["gs_E0"]) <= 1e-10 * abs(g["gs_E0"])
    af = CASES[tag][3]
    for spin_down in ((False, True) if af else (False,)):
        G = inst.Green_function(np.array(ZS), spin_down)
        for k in range(len(ZS)):
            ref = g[("gzdn" if spin_down else "gz") + str(k)]
            assert np.max(np.abs(G[k] - ref)) < 1e-9, (tag, spin_down, k)
    with pytest.raises(ValueError):
        inst.qmatrix()


def test_green_function_kernel_vs_numpy(pg):
    rng = np.random.default_rng(5)
    L, M = 12, 700
    e = np.sort(rng.uniform(-6, 6, M))
    v = rng.normal(size=(L, M)) + 1j * rng.normal(size=(L, M))
    zs = rng.uniform(-5, 5, 33) + 1j * rng.uniform(0.01, 2, 33)
    G = pg.green_function(e, v, zs)
    for w, z in enumerate(zs):
        ref = qo.green_function(e, v, z)
        assert np.max(np.abs(G[w] - ref)) < 1e-12 * np.max(np.abs(ref)) * 10


def test_large_sector_matvec_vs_oracle(pg):
    """3x4 cluster with t' at half filling (dim 853,776): engine vs oracle on
    the same seeded vector."""
    import models
    ns, nb, ops = models.hubbard_cluster(4, 3)
    params = {"t": 1.0, "tp": -0.3, "U": 8.0, "mu": 4.0}
    m = pg.ClusterModel(ns, nb)
    for name, (typ, els) in ops.items():
        m.new_operator(name, typ, els)
    H = pg.Hamiltonian(m, params, "R0:N12:S0")
    assert H.dim == 853776
    up, dn, pr = qo.combine_terms(ops, params, ns)
    S = qo.Sector(ns, 6, 6, up, dn, pr)
    x = qo.seeded_start(H.dim, 3)
    y = H.matvec(x)
    ref = S.matvec(x, nthreads=8)
    assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_errors(pg):
    m, params, sec = engine_model("chain8")
    with pytest.raises(ValueError):
        pg.Sector("R0:N7:S0")
    with pytest.raises(pg.QcmgError):
        pg.apply_c(8, 99, 1, 4, 4, np.zeros(4900))
    H = pg.Hamiltonian(m, params, sec)
    with pytest.raises(pg.QcmgError) as ei:
        H.lanczos(max_iter=3)
    assert ei.value.code == -4


@pytest.mark.parametrize("tag", ["chain8", "chain8_n7"])
def test_fixed_point_product_matches_reference(pg, tag):
    """The fixed-point product (hops +-t) against the reference's FP64 product."""
    g = load_golden(tag)
    m, params, sec = engine_model(tag)
    H = pg.Hamiltonian(m, params, sec)
    assert H.fx_available()
    x = g["h_x0"]
    ref = g["h_Hx0"]
    y = H.matvec(x)
    assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref))
    y2 = np.full(H.dim, 0.25)
    H.mult_add(x, y2)
    assert np.max(np.abs(y2 - 0.25 - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("mu", [4.0, 3.7])
@pytest.mark.parametrize("slabs", ["1", "2"])
@pytest.mark.parametrize("shape,n", [((4, 3), 12), ((13, 1), 10)])
def test_fixed_point_product_slab_variants(pg, monkeypatch, slabs, shape, n, mu):
    """Pass U with one and two slabs per round, on an even half basis (4x3,
    du = 924: 16-byte pass D loads) and an odd one (13-site chain, 5+5
    electrons, du = 1287: split bulk copies, 8-byte pass D loads), against
    the oracle on the same seeded vector.  mu = 4 gives small-integer
    diagonal energies (one 64-bit product per diagonal term), mu = 3.7 does
    not (128-bit products)."""
    import models
    monkeypatch.setenv("QCMG_FX_SLABS", slabs)
    ns, nb, ops = models.hubbard_cluster(*shape)
    params = {"t": 1.0, "U": 8.0, "mu": mu}
    m = pg.ClusterModel(ns, nb)
    for name, (typ, els) in ops.items():
        if name in params:
            m.new_operator(name, typ, els)
    H = pg.Hamiltonian(m, params, f"R0:N{n}:S0")
    assert H.fx_available()
    up, dn, pr = qo.combine_terms({k: v for k, v in ops.items() if k in params}, params, ns)
    S = qo.Sector(ns, n // 2, n // 2, up, dn, pr)
    x = qo.seeded_start(H.dim, 5)
    ref = S.matvec(x, nthreads=8)
    y = H.matvec(x)
    assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref))
    y2 = np.full(H.dim, -0.5)
    H.mult_add(x, y2)
    assert np.max(np.abs(y2 + 0.5 - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_fixed_point_not_used_for_mixed_hops(pg):
    m, params, sec = engine_model("ladder2x4_af")  # t and t' differ
    H = pg.Hamiltonian(m, params, sec)
    assert not H.fx_available()


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_fixed_point_conversion_roundtrip(pg):
    torch = _torch()
    from pyqcm_gb300 import _lib
    x = torch.randn(100003, dtype=torch.float64, device="cuda") * 1e-3
    x[7] = 0.0
    q = torch.empty(x.numel(), dtype=torch.int64, device="cuda")
    E, mb = _lib.c_int(), _lib.c_int()
    _lib.check(pg.lib().qcmg_fx_from_f64(x.numel(), x.data_ptr(), q.data_ptr(), E, mb, None))
    back = torch.empty_like(x)
    _lib.check(pg.lib().qcmg_fx_to_f64(x.numel(), q.data_ptr(), E.value, back.data_ptr(), None))
    err = float((back - x).abs().max())
    assert err <= 2.0 ** (E.value - 1) * 1.0000001
    assert err <= 2.0 ** -55 * float(x.abs().max())
    assert float(back[7]) == 0.0


def test_fixed_point_device_accumulate(pg):
    """qcmg_matvec_fx with QCMG_ACCUMULATE: y <- y + H x on device
    fixed-point vectors, against y0 + the reference's product (chain8)."""
    torch = _torch()
    from pyqcm_gb300 import _lib
    g = load_golden("chain8")
    m, params, sec = engine_model("chain8")
    H = pg.Hamiltonian(m, params, sec)
    x = torch.tensor(g["h_x0"], dtype=torch.float64, device="cuda")
    y0 = torch.linspace(-1.0, 1.0, H.dim, dtype=torch.float64, device="cuda")
    qx = torch.empty(H.dim, dtype=torch.int64, device="cuda")
    qy = torch.empty_like(qx)
    Ex, mbx, Ey, mby = _lib.c_int(), _lib.c_int(), _lib.c_int(), _lib.c_int()
    _lib.check(pg.lib().qcmg_fx_from_f64(H.dim, x.data_ptr(), qx.data_ptr(), Ex, mbx, None))
    _lib.check(pg.lib().qcmg_fx_from_f64(H.dim, y0.data_ptr(), qy.data_ptr(), Ey, mby, None))
    e = Ey.value
    for _ in range(2):  # two accumulations in a row
        e = H.matvec_fx_device(qx.data_ptr(), Ex.value, mbx.value, qy.data_ptr(), Ey_in=e)
    y = torch.empty_like(x)
    _lib.check(pg.lib().qcmg_fx_to_f64(H.dim, qy.data_ptr(), e, y.data_ptr(), None))
    torch.cuda.synchronize()
    ref = y0.cpu().numpy() + 2.0 * g["h_Hx0"]
    assert np.max(np.abs(y.cpu().numpy() - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_fixed_point_product_4x4_full_sector(pg):
    """4x4 Hubbard cluster, half filling (dim 165,636,900): fixed-point
    product against the FP64 product, both on the GPU, same vector."""
    torch = _torch()
    import models
    from pyqcm_gb300 import _lib
    ns, nb, ops = models.hubbard_cluster(4, 4)
    m = pg.ClusterModel(ns, nb)
    for name, (typ, els) in ops.items():
        m.new_operator(name, typ, els)
    H = pg.Hamiltonian(m, {"t": 1.0, "U": 8.0, "mu": 4.0}, "R0:N16:S0")
    assert H.dim == 165636900 and H.fx_available()
    gen = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn(H.dim, dtype=torch.float64, device="cuda", generator=gen)
    x /= torch.linalg.vector_norm(x)
    qx = torch.empty(H.dim, dtype=torch.int64, device="cuda")
    E, mb = _lib.c_int(), _lib.c_int()
    _lib.check(pg.lib().qcmg_fx_from_f64(H.dim, x.data_ptr(), qx.data_ptr(), E, mb, None))
    qy = torch.empty_like(qx)
    Ey = H.matvec_fx_device(qx.data_ptr(), E.value, mb.value, qy.data_ptr())
    y_fx = torch.empty_like(x)
    _lib.check(pg.lib().qcmg_fx_to_f64(H.dim, qy.data_ptr(), Ey, y_fx.data_ptr(), None))
    H.set_path(False)
    y64 = torch.empty_like(x)
    H.matvec_device(x.data_ptr(), y64.data_ptr())
    err = float((y_fx - y64).abs().max())
    assert err <= 1e-13 * float(y64.abs().max())
    del qx, qy, y_fx, y64, x
    torch.cuda.empty_cache()


def test_fixed_point_lanczos_long_run_stays_finite(pg):
    """700 Lanczos steps without convergence (tolerance 1e-300): the lazy
    vector scale must not drift out of double range; the run ends with
    NOCONV, not with a numerical breakdown."""
    m, params, sec = engine_model("chain8")
    H = pg.Hamiltonian(m, params, sec)
    assert H.fx_available()
    with pytest.raises(pg.QcmgError) as ei:
        H.lanczos(tol=1e-300, max_iter=700, reorth=0, want_psi=False)
    assert ei.value.code == -4, ei.value


def test_lanczos_4x4_full_sector_both_paths(pg):
    """4x4 Hubbard cluster, half filling (dim 165,636,900): ground-state
    energy to 1e-10 on the fixed-point path against the FP64 path (the
    reference's arithmetic), same seeded start."""
    _torch()
    import models
    ns, nb, ops = models.hubbard_cluster(4, 4)
    m = pg.ClusterModel(ns, nb)
    for name, (typ, els) in ops.items():
        m.new_operator(name, typ, els)
    H = pg.Hamiltonian(m, {"t": 1.0, "U": 8.0, "mu": 4.0}, "R0:N16:S0")
    e_fx, _, a_fx, _ = H.lanczos(tol=1e-10, max_iter=800, reorth=0, want_psi=False)
    H.set_path(False)
    e_64, _, a_64, _ = H.lanczos(tol=1e-10, max_iter=800, reorth=0, want_psi=False)
    assert np.isfinite(e_fx) and np.isfinite(e_64)
    assert abs(e_fx - e_64) <= 1e-10 * abs(e_64), (e_fx, e_64, len(a_fx), len(a_64))


def test_multidot_against_numpy(pg):
    torch = _torch()
    from pyqcm_gb300 import _lib
    gen = torch.Generator(device="cuda").manual_seed(11)
    n, m = 1_000_003, 7
    V = [torch.randn(n, dtype=torch.float64, device="cuda", generator=gen) for _ in range(m)]
    w = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
    ptrs = torch.tensor([v.data_ptr() for v in V], dtype=torch.int64, device="cuda")
    out = np.zeros(m)
    _lib.check(pg.lib().qcmg_multidot(m, ptrs.data_ptr(), w.data_ptr(), n, _lib.ptr(out), None))
    ref = np.array([float(torch.dot(v, w)) for v in V])
    assert np.max(np.abs(out - ref)) < 1e-12 * np.sqrt(n)
    out2 = np.zeros(m)
    _lib.check(pg.lib().qcmg_multidot(m, ptrs.data_ptr(), w.data_ptr(), n, _lib.ptr(out2), None))
    assert np.array_equal(out, out2)  # deterministic


@pytest.mark.parametrize("fixed_point", [True, False])
@pytest.mark.parametrize("offset", [0, 1])
def test_product_into_page_locked_host_vectors(pg, fixed_point, offset):
    """Products with a page-locked host y take the zero-copy path (x copied
    in, the result read-modify-written straight into y), pageable ones the
    staged copies.  Both against the oracle, accumulating and not, on a
    16-byte-aligned y and on one starting 8 bytes in (element-wise
    accesses)."""
    torch = _torch()
    import models
    from pyqcm_gb300 import _lib
    ns, nb, ops = models.hubbard_cluster(4, 3)
    params = {"t": 1.0, "U": 8.0, "mu": 4.0}
    m = pg.ClusterModel(ns, nb)
    for name, (typ, els) in ops.items():
        if name in params:
            m.new_operator(name, typ, els)
    H = pg.Hamiltonian(m, params, "R0:N12:S0")
    H.set_path(fixed_point)
    up, dn, pr = qo.combine_terms({k: v for k, v in ops.items() if k in params}, params, ns)
    S = qo.Sector(ns, 6, 6, up, dn, pr)
    x = qo.seeded_start(H.dim, 7)
    ref = S.matvec(x, nthreads=8)
    tol = 1e-13 * np.max(np.abs(ref))
    buf = torch.empty(H.dim + 1, dtype=torch.float64, pin_memory=True)
    y = buf.numpy()[offset:offset + H.dim]
    y[:] = 0.75
    H.mult_add(x, y)
    assert np.max(np.abs(y - 0.75 - ref)) <= tol
    y2 = np.full(H.dim, 0.75)  # pageable: staged copies
    H.mult_add(x, y2)
    assert np.max(np.abs(y2 - y)) <= tol
    y[:] = 3.0  # y = H x overwrites
    _lib.check(_lib.lib().qcmg_matvec(H._h, _lib.ptr(x), _lib.ptr(y), 0))
    assert np.max(np.abs(y - ref)) <= tol
