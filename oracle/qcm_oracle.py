"""CPU oracle for the exact-diagonalization hot path.  TEST INFRASTRUCTURE
ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it
as the checker; the product never imports it.

Restates pyqcm's algorithms with numpy/SciPy on top of the C arithmetic in
qcm_oracle.c (compiled on first use into oracle/_build):
  - combined factorized Hamiltonian of a value map (Hamiltonian_Factorized
    HS_ops_map / mult_add, src_ed/Hamiltonian/Hamiltonian_Factorized.hpp:50-87);
  - seeded start vector: std::default_random_engine(seed) with
    std::normal_distribution, normalized (src_util/vector_num.cpp:114-119);
  - Lanczos ground state without reorthogonalization, Ritz residual from the
    tridiagonal eigensystem (src_ed/Hamiltonian/Lanczos.hpp:41-143,
    Lanczos.cpp:25-52 -- dstev from LAPACK here too);
  - Freund band Lanczos with deflation and the p-step convergence test, and
    the Q-matrix Q = P U (src_ed/Hamiltonian/Lanczos.hpp:214-395,
    Hamiltonian_base.hpp:229-254);
  - Q-matrix assembly around a ground state: e -= E0, holes flipped, degenerate
    poles merged, particle part conjugated (src_ed/model_instance.hpp:711-817,
    src_ed/Q_matrix.hpp:180-291);
  - Lehmann Green function G(z) = V diag(1/(z-e)) V^dagger
    (src_ed/Q_matrix.hpp:133-151, src_util/VDVH_kernel.cpp:28-48).
Parity of this restatement is pinned against tests/golden (the reference's
own outputs).
"""
import ctypes
import math
import os
import subprocess

import numpy as np
import scipy.linalg as sla
from scipy.linalg import lapack

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
_LIB = None

u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def build():
    """Compiles qcm_oracle.c, lattice_oracle.c and qcm_oracle_rng.cpp into
    oracle/_build."""
    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "libqcm_oracle.so")
    srcs = [os.path.join(HERE, "qcm_oracle.c"), os.path.join(HERE, "lattice_oracle.c"),
            os.path.join(HERE, "qcm_oracle_rng.cpp")]
    if os.path.exists(so) and all(os.path.getmtime(so) >= os.path.getmtime(s) for s in srcs):
        return so
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        cc = "g++" if s.endswith(".cpp") else "gcc"
        subprocess.run([cc, "-O2", "-fPIC", "-fopenmp", "-c", s, "-o", o], check=True)
        objs.append(o)
    tmp = so + ".tmp"
    subprocess.run(["g++", "-shared", "-fopenmp", "-o", tmp] + objs, check=True)
    os.replace(tmp, so)
    return so


def lib():
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(build())
        L.qo_halfbasis.restype = ctypes.c_size_t
        L.qo_halfbasis.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.qo_halfop_build.restype = ctypes.c_size_t
        L.qo_halfop_build.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, i32p, i32p, f64p,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p]
        L.qo_matvec.restype = None
        L.qo_matvec.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, u32p, u32p,
                                u32p, u32p, f64p, f64p, u32p, u32p, f64p, f64p, ctypes.c_int,
                                i32p, i32p, f64p, f64p, f64p, ctypes.c_int]
        L.qo_apply_c.restype = None
        L.qo_apply_c.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, f64p, f64p, ctypes.c_double]
        L.qo_seeded_normal.restype = None
        L.qo_seeded_normal.argtypes = [ctypes.c_size_t, ctypes.c_uint, f64p]
        pp = ctypes.POINTER(ctypes.c_void_p)
        for name, args in (("qo_multidot", [ctypes.c_int, pp, f64p, ctypes.c_size_t, f64p,
                                             ctypes.c_int]),
                           ("qo_sub_rank1", [ctypes.c_int, pp, f64p, f64p, ctypes.c_size_t,
                                              ctypes.c_int]),
                           ("qo_sub_combination", [ctypes.c_int, pp, f64p, f64p,
                                                    ctypes.c_size_t, ctypes.c_int])):
            getattr(L, name).restype = None
            getattr(L, name).argtypes = args
        hop = [ctypes.c_int, f64p, ctypes.c_int, i32p, i32p, i32p, f64p]
        L.lo_sef_grid.restype = ctypes.c_double
        L.lo_sef_grid.argtypes = ([ctypes.c_int, ctypes.c_int, f64p, f64p, f64p] + hop
                                  + [ctypes.c_int] * 4)
        L.lo_cpt.restype = None
        L.lo_cpt.argtypes = ([ctypes.c_int, ctypes.c_int, f64p] + hop
                             + [ctypes.c_int, f64p, f64p, f64p, ctypes.c_int])
        L.lo_kmean.restype = None
        L.lo_kmean.argtypes = ([ctypes.c_int, ctypes.c_int, f64p] + hop
                               + [ctypes.c_int] * 3 + [ctypes.c_double, f64p, ctypes.c_int])
        _LIB = L
    return _LIB


# ----------------------------------------------------------------------------
# bases and operators


def halfbasis(L, N):
    if N < 0 or N > L:
        return np.zeros(0, np.uint32)
    n = lib().qo_halfbasis(L, N, None)
    out = np.zeros(n, np.uint32)
    lib().qo_halfbasis(L, N, out.ctypes.data)
    return out


def halfop(L, N, elements):
    """CSR (rowptr, col, val) of the hopping part and the diagonal of one spin,
    from elements (r, c, v) on orbitals 0..L-1 (both triangles given)."""
    el = list(elements)
    r = np.array([e[0] for e in el], np.int32)
    c = np.array([e[1] for e in el], np.int32)
    v = np.array([e[2] for e in el], np.float64)
    nnz = lib().qo_halfop_build(L, N, len(el), r, c, v, None, None, None, None)
    dim = len(halfbasis(L, N))
    rp = np.zeros(dim + 1, np.uint32)
    col = np.zeros(max(nnz, 1), np.uint32)
    val = np.zeros(max(nnz, 1), np.float64)
    diag = np.zeros(max(dim, 1), np.float64)
    lib().qo_halfop_build(L, N, len(el), r, c, v, rp.ctypes.data, col.ctypes.data,
                          val.ctypes.data, diag.ctypes.data)
    return rp, col[:nnz], val[:nnz], diag[:dim]


def combine_terms(ops, values, n_orb):
    """Sums the named operators with their coefficients into one list of hops
    per spin and one list of density-density pairs.  One-body elements keep
    r <= c and get their conjugate added, as the reference's one_body_operator
    does (src_ed/Operators/one_body_operator.hpp:62-71); interaction elements
    are ordered r <= c (src_ed/Operators/interaction_operator.hpp:40-45)."""
    hop = {}
    pairs = {}
    for name, coef in values.items():
        if name not in ops or coef == 0.0:
            continue
        typ, els = ops[name]
        for r, c, v in els:
            if typ == "interaction":
                key = (min(r, c), max(r, c))
                pairs[key] = pairs.get(key, 0.0) + coef * v
            else:
                if r > c:
                    continue
                hop[(r, c)] = hop.get((r, c), 0.0) + coef * v
                if r != c:
                    hop[(c, r)] = hop.get((c, r), 0.0) + coef * v
    up = [(r, c, v) for (r, c), v in sorted(hop.items()) if r < n_orb and c < n_orb]
    dn = [(r - n_orb, c - n_orb, v) for (r, c), v in sorted(hop.items())
          if r >= n_orb and c >= n_orb]
    mixed = [(r, c) for (r, c) in hop if (r < n_orb) != (c < n_orb)]
    if mixed:
        raise ValueError("spin-flip one-body terms do not factorize")
    pr = [(r, c, v) for (r, c), v in sorted(pairs.items())]
    return up, dn, pr


class Sector:
    """Factorized Hamiltonian of one (N_up, N_dn) sector."""

    def __init__(self, L, nup, ndn, hop_up, hop_dn, pairs):
        self.L, self.nup, self.ndn = L, nup, ndn
        self.bin_up, self.bin_dn = halfbasis(L, nup), halfbasis(L, ndn)
        self.du, self.dd = len(self.bin_up), len(self.bin_dn)
        self.dim = self.du * self.dd
        self.up = halfop(L, nup, hop_up)
        self.dn = halfop(L, ndn, hop_dn)
        self.pr = np.array([p[0] for p in pairs], np.int32)
        self.pc = np.array([p[1] for p in pairs], np.int32)
        self.pv = np.array([p[2] for p in pairs], np.float64)

    def mult_add(self, x, y, nthreads=1):
        """y += H x (in place)."""
        x = np.ascontiguousarray(x, np.float64)
        assert y.dtype == np.float64 and y.flags.c_contiguous and len(y) == self.dim
        if len(self.pr) == 0:
            pr, pc, pv = np.zeros(1, np.int32), np.zeros(1, np.int32), np.zeros(1)
        else:
            pr, pc, pv = self.pr, self.pc, self.pv
        lib().qo_matvec(self.L, self.du, self.dd, self.bin_up, self.bin_dn,
                        self.up[0], self.up[1] if len(self.up[1]) else np.zeros(1, np.uint32),
                        self.up[2] if len(self.up[2]) else np.zeros(1), self.up[3],
                        self.dn[0], self.dn[1] if len(self.dn[1]) else np.zeros(1, np.uint32),
                        self.dn[2] if len(self.dn[2]) else np.zeros(1), self.dn[3],
                        len(self.pr), pr, pc, pv, x, y, nthreads)
        return y

    def matvec(self, x, nthreads=1):
        y = np.zeros(self.dim)
        return self.mult_add(x, y, nthreads)


def seeded_start(dim, seed=0):
    """The reference's seeded random start vector, normalized."""
    x = np.zeros(dim)
    lib().qo_seeded_normal(dim, seed, x)
    return x * (1.0 / np.linalg.norm(x))


def apply_c(L, orb, pm, nup, ndn, x):
    """c_orb (pm=-1) or c^dagger_orb (pm=+1) applied to x; orb >= L is down."""
    spin = orb >= L
    nup2 = nup + (0 if spin else pm)
    ndn2 = ndn + (pm if spin else 0)
    n2 = len(halfbasis(L, nup2)) * len(halfbasis(L, ndn2))
    y = np.zeros(max(n2, 1))
    lib().qo_apply_c(L, orb, pm, nup, ndn, np.ascontiguousarray(x, np.float64), y, 1.0)
    return y[:n2]


# ----------------------------------------------------------------------------
# Krylov solvers (reference algorithms)


def tridiag_lowest(alpha, beta):
    """Lowest eigenvalue and eigenvector of the Lanczos tridiagonal matrix,
    via LAPACK dstev as the reference does (Lanczos.cpp:25-52)."""
    if len(alpha) == 1:
        return alpha[0], np.array([1.0])
    d, z, info = lapack.dstev(np.array(alpha), np.array(beta[: len(alpha) - 1]), compute_v=1)
    assert info == 0
    return d[0], z[:, 0]


def lanczos_eigenvalue(mult_add, x0, accur=1e-12, max_iter=1000):
    """Returns (alpha, beta, E0) of the reference's LanczosEigenvalue."""
    dim = len(x0)
    r = x0.copy()
    q = np.zeros(dim)
    alpha, beta = [], []
    ritz = 2 * accur
    e0 = None
    while ritz > accur:
        if beta:
            r *= 1.0 / beta[-1]
            q *= -beta[-1]
        mult_add(r, q)
        r, q = q, r
        a = float(q @ r)
        alpha.append(a)
        r -= a * q
        beta.append(float(np.linalg.norm(r)))
        e0, ev = tridiag_lowest(alpha, beta)
        ritz = abs(ev[-1] * beta[-1])
        if len(alpha) > max_iter:
            raise RuntimeError(f"Lanczos procedure exceeded {max_iter} iterations")
    return np.array(alpha), np.array(beta), e0


def lanczos_eigenvector(mult_add, x0, alpha, beta):
    """The reference's LanczosEigenvector: replays the recurrence."""
    _, ev = tridiag_lowest(list(alpha), list(beta))
    gs = x0 * ev[0]
    r = x0.copy()
    q = np.zeros(len(x0))
    for j in range(1, len(ev)):
        mult_add(r, q)
        q -= alpha[j - 1] * r
        r, q = q / beta[j - 1], -beta[j - 1] * r
        gs += ev[j] * r
    return gs


def _ptrs(vs):
    a = (ctypes.c_void_p * max(len(vs), 1))(*[v.ctypes.data for v in vs])
    return ctypes.cast(a, ctypes.POINTER(ctypes.c_void_p))


def _multidot(vs, w, nthreads):
    out = np.zeros(len(vs))
    if vs:
        lib().qo_multidot(len(vs), _ptrs(vs), w, len(w), out, nthreads)
    return out


def _sub_rank1(vs, coef, w, nthreads):
    if vs:
        lib().qo_sub_rank1(len(vs), _ptrs(vs), np.ascontiguousarray(coef, np.float64), w, len(w),
                           nthreads)


def _sub_combination(vs, coef, w, nthreads):
    if vs:
        lib().qo_sub_combination(len(vs), _ptrs(vs), np.ascontiguousarray(coef, np.float64), w,
                                 len(w), nthreads)


def band_lanczos(mult_add, phi, M0, accur_deflation=1e-7, accur_band=1e-12, max_iter_BL=600,
                 nthreads=1):
    """Freund's band Lanczos as in the reference (Lanczos.hpp:214-395).
    Returns (evalues, U, P, M) or None when no iteration was possible.  The
    independent dot products and updates of one step are batched (a
    projection on the p start vectors, the in-band orthogonalization against
    v_j, the recurrence's combination of the previous vectors) and run on
    `nthreads` threads."""
    p = len(phi)
    pc = p
    if M0 > max_iter_BL:
        M0 = max_iter_BL
    M0p = (M0 // p + 1) * p
    M0 = M0p - pc
    v = [None] * M0p
    t = np.zeros((M0, M0))
    P = np.zeros((p, M0))
    defl = np.zeros(M0, int)
    Idx = []
    for i in range(p):
        v[i] = np.array(phi[i], np.float64, copy=True)
    ev_old = 1e12
    j = 0
    phis = [np.ascontiguousarray(f, np.float64) for f in phi]
    # a vector is released once the band has moved past it (index below
    # j - pc and not deflated)
    while j < M0:
        z = math.sqrt(_multidot([v[j]], v[j], nthreads)[0])
        if z < accur_deflation:
            if j >= pc:
                Idx.append(j - pc)
                defl[j - pc] = 1
            pc -= 1
            if pc == 0:
                break
            for k in range(j, j + pc):
                v[k] = v[k + 1]
            v[j + pc] = None
            continue
        v[j] *= 1.0 / z
        if j >= pc:
            t[j, j - pc] = z
        P[:, j] = _multidot(phis, v[j], nthreads)
        band = [v[k] for k in range(j + 1, j + pc)]
        zz = _multidot(band, v[j], nthreads)
        _sub_rank1(band, zz, v[j], nthreads)
        for k in range(j + 1, j + pc):
            if k >= pc:
                t[j, k - pc] = zz[k - j - 1]
        w_new = np.zeros(len(v[j]))
        mult_add(v[j], w_new)
        k0 = j - pc if j > pc else 0
        for k in range(k0, j):
            t[k, j] = t[j, k]
        _sub_combination([v[k] for k in range(k0, j)], t[k0:j, j], w_new, nthreads)
        v[j + pc] = w_new
        for k in Idx:
            w = _multidot([v[k]], w_new, nthreads)[0]
            _sub_rank1([w_new], [w], v[k], nthreads)
            t[k, j] = w
        w = _multidot([v[j]], w_new, nthreads)[0]
        _sub_rank1([w_new], [w], v[j], nthreads)
        t[j, j] = w
        for k in Idx:
            t[j, k] = t[k, j]
        if j >= 4 * p and j % p == 0:
            evt = np.linalg.eigvalsh(t[:j, :j])
            test = abs(evt[0] - ev_old)
            ev_old = evt[0]
            if test < accur_band:
                break
        if k0 >= 1 and (k0 - 1) not in Idx:
            v[k0 - 1] = None
        j += 1
    M = j
    if j == 0:
        return None
    evals, U = np.linalg.eigh(t[:j, :j])
    return evals, U, P[:, :M], M


def build_Q_matrix(mult_add, phi, dim, nthreads=1):
    """(e, Q) with Q = P U restricted to the first p Lanczos vectors
    (Hamiltonian_base.hpp:229-254).  Q has shape (p, M)."""
    p = len(phi)
    if dim == 0 or p == 0:
        return np.zeros(0), np.zeros((p, 0))
    M = int(14 * p * math.log(1.0 * dim))
    res = band_lanczos(mult_add, phi, M, nthreads=nthreads)
    if res is None:
        return np.zeros(0), np.zeros((p, 0))
    evals, U, P, M = res
    k = min(p, M)
    return evals, P[:, :k] @ U[:k, :]


def streamline(e, v, wtol=1e-5, vtol=1e-10):
    """Merges degenerate poles (Q_matrix.hpp:180-223): v is (L, M)."""
    L, M = v.shape
    e2, cols = [], []
    i = 0
    while i < M:
        j = i + 1
        while j < M and abs(e[j] - e[i]) <= wtol:
            j += 1
        n = j - i
        if n == 1:
            col = v[:, i]
            if np.sum(np.abs(col) ** 2) >= vtol:
                e2.append(e[i])
                cols.append(col)
        else:
            Q = v[:, i:j]
            QQ = Q @ Q.conj().T
            d, Uq = np.linalg.eigh(QQ)
            for k in range(L):
                if d[k] > vtol:
                    e2.append(e[i])
                    cols.append(Uq[:, k] * math.sqrt(d[k]))
        i = j
    if not cols:
        return np.zeros(0), np.zeros((L, 0), v.dtype)
    return np.array(e2), np.array(cols).T


def green_function(e, v, z):
    """G(z)[a, b] = sum_i v[a,i] conj(v[b,i]) / (z - e_i), returned in the
    reference's layout G(b, a) (src_util/VDVH_kernel.cpp:28-48)."""
    u = 1.0 / (z - e)
    G = (v * u) @ v.conj().T  # G[a, b]
    return G.T.copy()


def qmatrix_for_state(mult_add_of, L_orb, nup, ndn, psi, E0, orbitals, spin_down=False,
                      nthreads=1):
    """Q-matrix (e, v) of one ground state: holes then particles, as
    model_instance::build_qmatrix assembles them.  `orbitals` are the
    Green-function orbitals (0..n_sites-1); `mult_add_of(nup, ndn)` returns
    the (mult_add, dim) of the Hamiltonian of that sector."""
    blocks_e, blocks_v = [], []
    for pm in (-1, 1):
        spin = 1 if spin_down else 0
        nup2 = nup + (0 if spin else pm)
        ndn2 = ndn + (pm if spin else 0)
        if min(nup2, ndn2) < 0 or max(nup2, ndn2) > L_orb:
            continue
        phi = [apply_c(L_orb, o + spin * L_orb, pm, nup, ndn, psi) for o in orbitals]
        mult_add, dim = mult_add_of(nup2, ndn2)
        if dim == 0:
            continue
        e, Q = build_Q_matrix(mult_add, phi, dim, nthreads)
        e = e - E0
        if pm == -1:
            e = -e
        # streamline expects increasing energies, as in the reference
        e, Q = streamline(e, Q.astype(np.float64))
        if pm == 1:
            Q = Q.conj()
        blocks_e.append(e)
        blocks_v.append(Q)
    e = np.concatenate(blocks_e)
    v = np.concatenate(blocks_v, axis=1)
    return e, v


# ----------------------------------------------------------------------------
# Continued-fraction Green function (GF_method 'F')


def lanczos_green(mult_add, psi, accur=0.01, max_iter=400):
    """(a, b) of the reference's LanczosGreen (Lanczos.hpp:156-183): the
    three-term recurrence from the normalized psi, stopped when the product
    of the b's or the last b falls to accur, or after max_iter steps; b
    starts with 1 and has one entry more than a."""
    psi = np.array(psi, np.float64)
    q = np.zeros(len(psi))
    a, b = [], [1.0]
    prod = 1.0
    while prod > accur and abs(b[-1]) > accur and len(a) < max_iter:
        if a:  # psi <- q / beta, q <- -beta psi (vector_num.hpp:274-282)
            beta = b[-1]
            psi, q = q * (1.0 / beta), -beta * psi
        mult_add(psi, q)
        z = float(psi @ q)
        a.append(z)
        q -= z * psi
        zz = float(np.linalg.norm(q))
        b.append(zz)
        prod *= abs(zz)
    return np.array(a), np.array(b)


def continued_fraction(a, b, e0, norm, create):
    """The reference's continued_fraction(a, b, e0, norm, create)
    (continued_fraction.cpp:30-37): b -> b^2 with b[0] = norm, a shifted by
    the ground-state energy (electron part a - e0, hole part e0 - a)."""
    a = np.array(a, np.float64)
    b = np.array(b, np.float64) ** 2
    b[0] = norm
    a = a - e0 if create else e0 - a
    return a, b


def cf_evaluate(a, b, z):
    """G(z) = b0 / (z - a0 - b1 / (z - a1 - ...)) (continued_fraction.cpp:48-53)."""
    G = 0.0 + 0.0j
    for i in range(len(a) - 1, -1, -1):
        G = b[i] / (z - a[i] - G)
    return G


def cf_green_function_for_state(mult_add_of, L_orb, nup, ndn, psi, E0, weight, orbitals, zs,
                                spin_down=False, accur=0.01, max_iter=400):
    """G(z) of one ground state by continued fractions, real case, as
    model_instance<double>::build_cf (model_instance.cpp:35-100) and
    continued_fraction_set::Green_function (continued_fraction_set.cpp:63-98)
    assemble it: a fraction per orbital pair (o2 <= o1) from c_o1 psi
    (+ c_o2 psi), electron and hole parts; off-diagonal elements
    0.5 (G_{o1+o2} - G_o1o1 - G_o2o2).  Returns (nz, L, L)."""
    n = len(orbitals)
    spin = 1 if spin_down else 0
    frac = {}
    for pm in (-1, 1):
        nup2 = nup + (0 if spin else pm)
        ndn2 = ndn + (pm if spin else 0)
        if min(nup2, ndn2) < 0 or max(nup2, ndn2) > L_orb:
            continue
        mult_add, dim = mult_add_of(nup2, ndn2)
        if dim == 0:
            continue
        for i1, o1 in enumerate(orbitals):
            for i2 in range(i1 + 1):
                o2 = orbitals[i2]
                x = apply_c(L_orb, o1 + spin * L_orb, pm, nup, ndn, psi)
                if i2 != i1:
                    x = x + apply_c(L_orb, o2 + spin * L_orb, pm, nup, ndn, psi)
                norm = float(x @ x)
                if norm > 1e-14:
                    a, b = lanczos_green(mult_add, x / np.sqrt(norm), accur, max_iter)
                    frac[(pm, i1, i2)] = continued_fraction(a, b, E0, norm * weight, pm == 1)
    zs = np.atleast_1d(np.asarray(zs, np.complex128))
    G = np.zeros((len(zs), n, n), np.complex128)
    for w, z in enumerate(zs):
        def part(i1, i2):
            return sum(cf_evaluate(*frac[(pm, i1, i2)], z) for pm in (-1, 1) if (pm, i1, i2) in frac)
        d = [part(i, i) for i in range(n)]
        for i in range(n):
            G[w, i, i] = d[i]
        for i1 in range(n):
            for i2 in range(i1):
                t = 0.5 * (part(i1, i2) - d[i1] - d[i2])
                G[w, i1, i2] = G[w, i2, i1] = t
    return G


# ----------------------------------------------------------------------------
# Matrix continued-fraction Green function (GF_method 'M')


def _lowest_banded(A, B, p):
    """Lowest eigenvalue of the block-tridiagonal matrix with diagonal blocks
    A[j] and sub-diagonal blocks B[j] (LAPACK band eigensolver)."""
    from scipy.linalg import eigvals_banded
    m = len(A)
    sz = m * p
    bw = 2 * p - 1
    ab = np.zeros((bw + 1, sz))  # lower band: ab[r - c, c]
    for jj in range(m):
        for r in range(p):
            for c in range(p):
                if r >= c:
                    ab[r - c, jj * p + c] = A[jj][r, c]
                if jj < m - 1:
                    ab[p + r - c, jj * p + c] = B[jj][r, c]
    return float(eigvals_banded(ab, lower=True, select="i", select_range=(0, 0))[0])


def block_lanczos_svd(mult_add, q, M0, accur_deflation=1e-7, accur_band=1e-12, max_iter_BL=600):
    """(A, B) of the reference's blockLanczosSVD (Lanczos.hpp:603-790): the
    block recurrence H Q_j = Q_{j-1} B_{j-1} + Q_j A_j + Q_{j+1} B_j with B_j
    the symmetric square root of the residual's Gram matrix; convergence of
    the lowest eigenvalue of the block-tridiagonal matrix every p steps from
    step 2p, singular coupling blocks (eigenvalue of the Gram matrix below
    accur_deflation^2) stop the recurrence."""
    p = len(q)
    M0 = min(M0, max_iter_BL)
    Qc = [np.array(v, np.float64) for v in q]
    for l in range(p):  # the block is orthonormalized once more
        for k in range(l):
            Qc[l] = Qc[l] - float(Qc[k] @ Qc[l]) * Qc[k]
        nrm = float(np.linalg.norm(Qc[l]))
        if nrm < accur_deflation:
            raise RuntimeError("block Lanczos: rank-deficient start block")
        Qc[l] = Qc[l] / nrm
    Qp = None
    A, B = [], []
    ev_old = 1e12
    for j in range(M0):
        Z = []
        for k in range(p):
            z = np.zeros(len(Qc[k]))
            mult_add(Qc[k], z)
            Z.append(z)
        Aj = np.array([[float(Qc[k] @ Z[l]) for l in range(p)] for k in range(p)])
        Aj = np.triu(Aj) + np.triu(Aj, 1).T  # computed for k <= l, mirrored
        A.append(Aj)
        for l in range(p):
            for k in range(p):
                Z[l] = Z[l] - Aj[k, l] * Qc[k]
        if j > 0:
            Bp = B[-1]
            for l in range(p):
                for k in range(p):
                    Z[l] = Z[l] - Bp[l, k] * Qp[k]
        G = np.array([[float(Z[k] @ Z[l]) for l in range(p)] for k in range(p)])
        G = np.triu(G) + np.triu(G, 1).T
        D, V = np.linalg.eigh(G)
        singular = bool(np.any(D < accur_deflation ** 2))
        B.append((V * np.sqrt(np.maximum(D, 0.0))) @ V.T)
        if singular:
            break
        Binv = (V / np.sqrt(D)) @ V.T
        Qn = [sum(Binv[k, l] * Z[k] for k in range(p)) for l in range(p)]
        Qp, Qc = Qc, Qn
        if j + 1 >= 2 * p and (j + 1) % p == 0:
            e0 = _lowest_banded(A, B, p)
            delta = abs(e0 - ev_old)
            ev_old = e0
            if delta < accur_band:
                break
    return A, B


def mcf_evaluate(A, B, W, z):
    """G(z) = W^T F_0 W with F_M = 0, F_j = (z - A_j - B_j^T F_{j+1} B_j)^-1
    (matrix_continued_fraction.hpp:139-185; the last B is not used)."""
    p = A[0].shape[0]
    F = np.zeros((p, p), np.complex128)
    M = len(A)
    for j in range(M - 1, -1, -1):
        S = B[j].T @ F @ B[j] if j < M - 1 else 0.0
        F = np.linalg.inv(z * np.eye(p) - A[j] - S)
    return W.T @ F @ W


def mcf_green_function_for_state(mult_add_of, L_orb, nup, ndn, psi, E0, weight, orbitals, zs,
                                 spin_down=False, accur_deflation=1e-7):
    """G(z) of one ground state by matrix continued fractions, real case, as
    model_instance::build_mcf (model_instance.hpp:847-955) and
    mcf_set::Green_function (mcf_set.hpp:112-130) form it: per part
    (pm = -1 holes, +1 electrons) the start block c_o psi, its Gram-Schmidt
    factor W (times sqrt(weight)), block Lanczos on the orthonormal block, and
    the shifted fraction; G = G_e + G_h^T.  Returns (nz, L, L)."""
    spin = 1 if spin_down else 0
    parts = []
    for pm in (-1, 1):
        nup2 = nup + (0 if spin else pm)
        ndn2 = ndn + (pm if spin else 0)
        if min(nup2, ndn2) < 0 or max(nup2, ndn2) > L_orb:
            continue
        mult_add, dim = mult_add_of(nup2, ndn2)
        if dim == 0:
            continue
        phi = [apply_c(L_orb, o + spin * L_orb, pm, nup, ndn, psi) for o in orbitals]
        p = len(phi)
        q = [v.copy() for v in phi]
        W = np.zeros((p, p))
        pa = p
        for l in range(p):
            for k in range(l):
                z = float(q[k] @ q[l])
                W[k, l] = z
                q[l] = q[l] - z * q[k]
            nrm = float(np.linalg.norm(q[l]))
            if nrm < accur_deflation:
                pa = l
                break
            W[l, l] = nrm
            q[l] = q[l] / nrm
        if pa == 0:
            continue
        W = W[:pa] * np.sqrt(weight)
        A, B = block_lanczos_svd(mult_add, q[:pa], int(14 * pa * np.log(1.0 * dim)))
        A = [a - E0 * np.eye(pa) if pm == 1 else E0 * np.eye(pa) - a for a in A]
        parts.append((pm, A, B, W))
    zs = np.atleast_1d(np.asarray(zs, np.complex128))
    G = np.zeros((len(zs), len(orbitals), len(orbitals)), np.complex128)
    for w, z in enumerate(zs):
        for pm, A, B, W in parts:
            g = mcf_evaluate(A, B, W, z)
            G[w] += g if pm == 1 else g.T
    return G
