"""CPU oracle for the lattice integrals (CPT spectral function, VCA
Potthoff functional, CDMFT projected Green function).  TEST INFRASTRUCTURE
ONLY: tests and bench.py's CPU-baseline legs use it as the checker; the
product never imports it.

numpy builds the per-frequency pieces (pyqcm's formulas, cited below); the
per-(K, z) work runs in lattice_oracle.c (LU with partial pivoting, OpenMP
over K rows, sums in a fixed order).  Inputs are the cluster's Lehmann data
(e, v), the bath (tcb, eb) and the lattice hopping in Fourier form (R, the
inter-cluster elements, H - H_c, orbital positions), as
LatticeModel.fourier() and the cluster solve give them; the Fourier data
are pinned against the reference's own t(k) by the lattice Fourier tests.
"""
import numpy as np

from qcm_oracle import lib


def green(e, v, zs):
    """G(z)_ab = sum_i v_ai conj(v_bi) / (z - e_i) for every z of zs
    (src_ed/Q_matrix.hpp:133-151): (nz, L, L)."""
    zs = np.atleast_1d(np.asarray(zs, np.complex128))
    d = 1.0 / (zs[:, None] - np.asarray(e, np.float64)[None, :])
    v = np.asarray(v, np.complex128)
    return np.einsum("ai,zi,bi->zab", v, d, v.conj(), optimize=True)


def gamma(tcb, eb, zs):
    """Gamma(z) = tcb diag(1/(z - eb)) tcb^+ (src_ed/model_instance.hpp:
    425-475 with the bath diagonal): (nz, L, L)."""
    zs = np.atleast_1d(np.asarray(zs, np.complex128))
    tcb = np.asarray(tcb, np.complex128)
    L = tcb.shape[0]
    if tcb.size == 0:
        return np.zeros((len(zs), L, L), np.complex128)
    d = 1.0 / (zs[:, None] - np.asarray(eb, np.float64)[None, :])
    return np.einsum("ai,zi,bi->zab", tcb, d, tcb.conj())


def base(states, tcb, eb, hdiff, zs):
    """Base(z) = G(z)^-1 + Gamma(z) - (H - H_c) and log|det G(z)| per z
    (src_qcm/CPT.cpp:22-86): states = [(e, v, weight), ...] (Lehmann data
    of the kept cluster states, v of shape (L, M))."""
    zs = np.atleast_1d(np.asarray(zs, np.complex128))
    G = sum(w * green(e, v, zs) for e, v, w in states)
    B = np.linalg.inv(G) + gamma(tcb, eb, zs) - np.asarray(hdiff)[None]
    ldg = np.linalg.slogdet(G)[1]
    return np.ascontiguousarray(B), np.ascontiguousarray(ldg, np.float64)


def _hops(R, els):
    R = np.ascontiguousarray(np.asarray(R, np.float64).reshape(-1, 3))
    er = np.ascontiguousarray([e[0] for e in els], np.int32)
    ec = np.ascontiguousarray([e[1] for e in els], np.int32)
    en = np.ascontiguousarray([e[2] for e in els], np.int32)
    ev = np.ascontiguousarray(np.array([e[3] for e in els], np.complex128)).view(np.float64)
    return [len(R), R, len(els), er, ec, en, ev]


def sef_grid(B, ldg, wt, R, els, grid, nthreads=1):
    """sum_w wt_w (1/N_K) sum_K log|det(V G - 1)| on the K grid (gx, gy, gz)
    (lattice_model_instance.cpp:503-584, 624-643), frequencies i w with
    Base B (nw, L, L) and log|det G| ldg."""
    L = B.shape[1]
    return lib().lo_sef_grid(L, B.shape[0], B.view(np.float64).reshape(-1),
                             np.ascontiguousarray(ldg, np.float64),
                             np.ascontiguousarray(wt, np.float64), *_hops(R, els), *grid,
                             nthreads)


def cpt(B, R, els, K, gpos, nthreads=1):
    """Periodized CPT Green function g(K, z): (nz, nk) complex for K in the
    reduced basis (nk x 3) (CPT.cpp:76-86, lattice_model.cpp:724-740)."""
    K = np.ascontiguousarray(np.asarray(K, np.float64).reshape(-1, 3))
    g = np.zeros(2 * B.shape[0] * len(K))
    lib().lo_cpt(B.shape[1], B.shape[0], B.view(np.float64).reshape(-1), *_hops(R, els), len(K),
                 K, np.ascontiguousarray(gpos, np.float64).reshape(-1), g, nthreads)
    return g.view(np.complex128).reshape(B.shape[0], len(K))


def kmean(B, R, els, grid, off=0.5, nthreads=1):
    """(1/N_K) sum_K M(K, z)^-1 per frequency on the grid K = (i + off)/g
    (the CDMFT projected Green function, CPT.cpp:283-345): (nw, L, L)."""
    L = B.shape[1]
    out = np.zeros(2 * B.shape[0] * L * L)
    lib().lo_kmean(L, B.shape[0], B.view(np.float64).reshape(-1), *_hops(R, els), *grid, off,
                   out, nthreads)
    return out.view(np.complex128).reshape(B.shape[0], L, L)


# ----------------------------------------------------------------------------
# the cluster side, from the operators of a cluster model


def one_body_blocks(ops, values, n_orb, n_sites, spin_down=False):
    """(tc, tcb, eb) of one spin block: the one-body matrix of the value map
    (elements keep r <= c, the conjugate of r < c added,
    src_ed/Operators/one_body_operator.hpp:62-71), split into cluster,
    cluster-bath and bath parts, the bath diagonalized when it is not
    diagonal (src_ed/model_instance.hpp:425-475)."""
    T = np.zeros((2 * n_orb, 2 * n_orb), np.complex128)
    for name, (typ, els) in ops.items():
        coef = values.get(name, 0.0)
        if typ != "one-body" or coef == 0.0:
            continue
        for r, c, v in els:
            T[r, c] += coef * v
            if r != c:
                T[c, r] += np.conj(coef * v)
    o = n_orb if spin_down else 0
    B = T[o:o + n_orb, o:o + n_orb]
    tc, tcb, tb = B[:n_sites, :n_sites], B[:n_sites, n_sites:], B[n_sites:, n_sites:]
    if tb.size and np.count_nonzero(tb - np.diag(np.diag(tb))):
        d, S = np.linalg.eigh(tb)
        return tc, tcb @ S, d
    return tc, tcb, np.diag(tb).real.copy()


def cluster_lehmann(ops, values, n_orb, n_sites, sector, spins=(False,), nthreads=1, seed=0):
    """The cluster's ground state in one sector (Lanczos from the seeded start)
    and the Q-matrix of each requested spin block (band Lanczos):
    (E0, {spin_down: (e, v)}), v of shape (n_sites, M)."""
    import qcm_oracle as qo
    up, dn, pr = qo.combine_terms(ops, values, n_orb)
    parts = dict((p[0], int(p[1:])) for p in sector.split(":"))
    N, Sz = parts["N"], parts["S"]
    nup, ndn = (N + Sz) // 2, (N - Sz) // 2
    sectors = {}

    def mao(nu, nd):
        if (nu, nd) not in sectors:
            sectors[(nu, nd)] = qo.Sector(n_orb, nu, nd, up, dn, pr)
        s = sectors[(nu, nd)]
        return (lambda x, y: s.mult_add(x, y, nthreads)), s.dim

    ma, dim = mao(nup, ndn)
    x0 = qo.seeded_start(dim, seed)
    al, be, e0 = qo.lanczos_eigenvalue(ma, x0)
    psi = qo.lanczos_eigenvector(ma, x0, al, be)
    return e0, {sd: qo.qmatrix_for_state(mao, n_orb, nup, ndn, psi, e0, range(n_sites), sd,
                                              nthreads)
                for sd in spins}


def cdmft_host(states, tcb, eb, hdiff, R, els, wn, kside, dimk, nthreads=1):
    """G_host(i w) = P^-1 + Sigma + t_c - i w = P^-1 - G^-1 - Gamma, with P the
    projected Green function on the kside^dimk midpoint grid
    (src_qcm/CPT.cpp:283-424): (nw, L, L)."""
    zs = 1j * np.asarray(wn, np.float64)
    B, _ = base(states, tcb, eb, hdiff, zs)
    grid = tuple(kside if dimk > d else 1 for d in range(3))
    P = kmean(B, R, els, grid, 0.5, nthreads)
    G = sum(w * green(e, v, zs) for e, v, w in states)
    return np.linalg.inv(P) - np.linalg.inv(G) - gamma(tcb, eb, zs)


def bath_fit(ops, values, names, n_orb, n_sites, host, wn, weights, x0, spin_down=False,
             xtol=1e-6, ftol=1e-8):
    """The bath fit of one CDMFT step: SciPy least_squares ('trf', Jacobian
    by differences) of sqrt(weight) (Gamma(i w; x) + G_host(i w)) over the
    cluster parameters `names` (pyqcm/cdmft.py:1539-1640,
    src_qcm/CPT.cpp:519-555).  Returns the fitted x."""
    import scipy.optimize
    zs = 1j * np.asarray(wn, np.float64)
    sw = np.sqrt(np.asarray(weights, np.float64))[:, None, None]

    def resid(x):
        vals = dict(values)
        vals.update(zip(names, x))
        _, tcb, eb = one_body_blocks(ops, vals, n_orb, n_sites, spin_down)
        d = (gamma(tcb, eb, zs) + host) * sw
        return np.concatenate([d.real.ravel(), d.imag.ravel()])

    return scipy.optimize.least_squares(resid, np.asarray(x0, np.float64), method="trf",
                                        xtol=xtol, ftol=ftol, gtol=1e-12).x


def cdmft_distance(ops, values, names, x, n_orb, n_sites, host, wn, weights, normal=True,
                   spin_down=False):
    """The CDMFT distance at bath x: sum_w weight |Gamma(i w; x) + G_host(i w)|^2
    dw / dim^2, doubled for normal mixing (src_qcm/CPT.cpp:519-555)."""
    vals = dict(values)
    vals.update(zip(names, x))
    _, tcb, eb = one_body_blocks(ops, vals, n_orb, n_sites, spin_down)
    wn = np.asarray(wn, np.float64)
    d = gamma(tcb, eb, 1j * wn) + host
    dist = float(np.sum(np.asarray(weights)[:, None, None] * np.abs(d) ** 2))
    if normal:
        dist *= 2.0
    return dist * (wn[1] - wn[0]) / (host.shape[1] ** 2)
