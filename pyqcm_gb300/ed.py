"""Cluster exact-diagonalization layer on the GPU engine.

Mirrors the part of pyqcm's ED interface that sits on the factorized hot
path, with the same names and argument meanings:
  ClusterModel      ~ ED::new_model / ED::new_operator (src_ed/qcm_ED.hpp:34-78)
  Hamiltonian       ~ Hamiltonian<HF> in a new format 'G'
                      (src_ed/Hamiltonian/Hamiltonian_base.hpp:43-82):
                      mult_add, states, GS_energy, build_Q_matrix
  ModelInstance     ~ model_instance<HF> (src_ed/model_instance.hpp):
                      ground_state (low_energy_states), Green_function_solve
                      (build_qmatrix), Green_function, qmatrix,
                      hybridization_function, self_energy, Potthoff_functional
Every vector operation runs in libqcmg (no CPU fallback); the host keeps the
small dense pieces (Q-matrix assembly, hopping matrices).
"""
import math

import numpy as np

from . import _lib
from ._lib import QcmgError, as_f64, check, lib, ptr

# Global parameters with the reference's defaults (src_util/global_parameter.cpp:17-90).
GLOBAL = {
    "accur_lanczos": 1e-12,
    "max_iter_lanczos": 1000,
    "accur_band_lanczos": 1e-12,
    "accur_deflation": 1e-7,
    "max_iter_BL": 600,
    "accur_Q_matrix": 1e-5,
    "Qmatrix_wtol": 1e-5,
    "Qmatrix_vtol": 1e-10,
    "minimum_weight": 0.01,
    "temperature": 0.0,
    "seed": 0,
    "Lanczos_reorth": 0,
    # Green-function representation: 'L' Lehmann form from band Lanczos, 'F'
    # continued fractions, 'M' matrix continued fractions (block Lanczos)
    # (src_util/global_parameter.cpp:61,76,90)
    "GF_method": "L",
    "accur_continued_fraction": 0.01,
    "max_iter_CF": 400,
}
MIN_GAP = 1.0e-6      # src_ed/model.hpp:19
SMALL_VALUE = 1e-12   # degeneracy threshold of compute_weights


def set_global_parameter(name, value):
    if name not in GLOBAL:
        raise ValueError(f"unknown global parameter {name}")
    GLOBAL[name] = type(GLOBAL[name])(value)


class Sector:
    """Sector "R0:N8:S0": N electrons, S = 2 Sz (src_ed/sector.hpp:36-95)."""

    def __init__(self, s):
        parts = dict((p[0], int(p[1:])) for p in s.split(":"))
        if parts.get("R", 0) != 0:
            raise ValueError("the factorized format has a trivial point group: only R0 sectors")
        self.N, self.S = parts["N"], parts["S"]
        if (self.N + self.S) % 2:
            raise ValueError(f"invalid sector {s}")
        self.nup, self.ndn = (self.N + self.S) // 2, (self.N - self.S) // 2

    @staticmethod
    def of(nup, ndn):
        return Sector(f"R0:N{nup + ndn}:S{nup - ndn}")

    def name(self):
        return f"R0:N{self.N}:S{self.S}"

    def __repr__(self):
        return self.name()


class ClusterModel:
    """Cluster (impurity) model: n_sites cluster orbitals + n_bath bath
    orbitals; spin-orbital r < n_orb is up, r >= n_orb is down."""

    def __init__(self, n_sites, n_bath=0, name="clus"):
        self.name, self.n_sites, self.n_bath = name, n_sites, n_bath
        self.n_orb = n_sites + n_bath
        if self.n_orb > 32:
            raise ValueError("at most 32 orbitals per spin")
        self.operators = {}

    def new_operator(self, name, op_type, elements):
        if op_type not in ("one-body", "interaction"):
            raise ValueError("only one-body and density-density interaction operators factorize")
        self.operators[name] = (op_type, [(int(r), int(c), float(v)) for r, c, v in elements])

    def combine(self, values):
        """Hops per spin and density-density pairs of the value map.  One-body
        elements keep r <= c and add the conjugate of r < c
        (src_ed/Operators/one_body_operator.hpp:62-71)."""
        hop, pairs = {}, {}
        n = self.n_orb
        for name, coef in values.items():
            if name not in self.operators or coef == 0.0:
                continue
            typ, els = self.operators[name]
            for r, c, v in els:
                if typ == "interaction":
                    key = (min(r, c), max(r, c))
                    pairs[key] = pairs.get(key, 0.0) + coef * v
                elif r <= c:
                    hop[(r, c)] = hop.get((r, c), 0.0) + coef * v
                    if r != c:
                        hop[(c, r)] = hop.get((c, r), 0.0) + coef * v
        up, dn = [], []
        for (r, c), v in sorted(hop.items()):
            if r < n and c < n:
                up.append((r, c, v))
            elif r >= n and c >= n:
                dn.append((r - n, c - n, v))
            else:
                raise ValueError("spin-flip terms do not factorize")
        return up, dn, [(r, c, v) for (r, c), v in sorted(pairs.items())]

    def one_body_matrix(self, values, spin_down=False):
        up, dn, _ = self.combine(values)
        T = np.zeros((self.n_orb, self.n_orb))
        for r, c, v in (dn if spin_down else up):
            T[r, c] += v
        return T


def _arrays(els):
    r = np.array([e[0] for e in els], np.int32)
    c = np.array([e[1] for e in els], np.int32)
    v = np.array([e[2] for e in els], np.float64)
    return r, c, v


class State:
    def __init__(self, sector, energy, psi):
        self.sec, self.energy, self.psi = sector, energy, psi
        self.weight = 1.0
        self.gf = None
        self.gf_down = None


class Hamiltonian:
    """Factorized Hamiltonian of one sector on the GPU (format 'G')."""

    def __init__(self, model, values, sector):
        self.model = model
        self.sec = sector if isinstance(sector, Sector) else Sector(sector)
        up, dn, pairs = model.combine(values)
        L = model.n_orb
        ur, uc, uv = _arrays(up)
        dr, dc, dv = _arrays(dn)
        pr, pc, pv = _arrays(pairs)
        h = _lib.vp()
        check(lib().qcmg_hamiltonian_create(L, self.sec.nup, self.sec.ndn,
                                            len(up), ptr(ur), ptr(uc), ptr(uv),
                                            len(dn), ptr(dr), ptr(dc), ptr(dv),
                                            len(pairs), ptr(pr), ptr(pc), ptr(pv), h))
        self._h = h
        du, dd, dim = _lib.c_size_t(), _lib.c_size_t(), _lib.c_size_t()
        check(lib().qcmg_hamiltonian_dims(h, du, dd, dim))
        self.dim_up, self.dim_dn, self.dim = du.value, dd.value, dim.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.qcmg_hamiltonian_destroy(h)
            self._h = None

    def mult_add(self, x, y):
        """y += H x (host numpy vectors, y modified in place)."""
        x = as_f64(x)
        assert y.dtype == np.float64 and y.flags.c_contiguous and y.shape == (self.dim,)
        check(lib().qcmg_matvec(self._h, ptr(x), ptr(y), _lib.QCMG_ACCUMULATE))

    def matvec(self, x):
        y = np.zeros(self.dim)
        check(lib().qcmg_matvec(self._h, ptr(as_f64(x)), ptr(y), 0))
        return y

    def matvec_device(self, x_ptr, y_ptr, accumulate=False, asynchronous=False):
        """y (+)= H x on device pointers (e.g. torch CUDA tensors' data_ptr())."""
        flags = _lib.QCMG_DEVICE_PTRS | (_lib.QCMG_ACCUMULATE if accumulate else 0)
        if asynchronous:
            flags |= _lib.QCMG_ASYNC
        check(lib().qcmg_matvec(self._h, x_ptr, y_ptr, flags))

    def set_stream(self, stream_ptr):
        """Launch on a caller-owned cudaStream_t (int handle, 0 = own stream)."""
        check(lib().qcmg_hamiltonian_set_stream(self._h, stream_ptr or None))

    def set_path(self, fixed_point):
        """True: fixed-point fast path where it applies (default); False: FP64."""
        check(lib().qcmg_hamiltonian_set_path(self._h, 1 if fixed_point else 0))

    def fx_available(self):
        a = _lib.c_int()
        check(lib().qcmg_hamiltonian_fx_available(self._h, a))
        return bool(a.value)

    def matvec_fx_device(self, qx_ptr, Ex, mbx, qy_ptr, asynchronous=False, Ey_in=None):
        """y = H x on fixed-point device vectors (y = y + H x when Ey_in, the
        exponent of the input y, is given); returns the exponent of y."""
        Ey = _lib.c_int(0 if Ey_in is None else Ey_in)
        flags = (_lib.QCMG_ASYNC if asynchronous else 0) | (0 if Ey_in is None else _lib.QCMG_ACCUMULATE)
        check(lib().qcmg_matvec_fx(self._h, qx_ptr, Ex, mbx, qy_ptr, Ey, flags))
        return Ey.value

    def halfop(self, spin):
        nnz = _lib.c_size_t()
        check(lib().qcmg_hamiltonian_halfop(self._h, spin, nnz, None, None, None, None))
        dim = self.dim_dn if spin else self.dim_up
        rp = np.zeros(dim + 1, np.uint32)
        col = np.zeros(max(nnz.value, 1), np.uint32)
        val = np.zeros(max(nnz.value, 1))
        diag = np.zeros(max(dim, 1))
        check(lib().qcmg_hamiltonian_halfop(self._h, spin, nnz, ptr(rp), ptr(col), ptr(val),
                                            ptr(diag)))
        return rp, col[: nnz.value], val[: nnz.value], diag[:dim]

    def lanczos(self, x0=None, tol=None, max_iter=None, reorth=None, want_psi=True):
        """Returns (E0, psi, alpha, beta)."""
        tol = GLOBAL["accur_lanczos"] if tol is None else tol
        max_iter = GLOBAL["max_iter_lanczos"] if max_iter is None else max_iter
        reorth = GLOBAL["Lanczos_reorth"] if reorth is None else reorth
        cap = max_iter + 2
        alpha, beta = np.zeros(cap), np.zeros(cap)
        psi = np.zeros(self.dim) if want_psi else None
        e0, nit = _lib.c_double(), _lib.c_int()
        x0a = None if x0 is None else as_f64(x0)
        check(lib().qcmg_lanczos_ground_state(self._h, ptr(x0a), GLOBAL["seed"], tol, max_iter,
                                              reorth, e0, ptr(psi), nit, ptr(alpha), ptr(beta),
                                              cap))
        n = nit.value
        if reorth:  # restarted runs return the last cycle's coefficients
            n = self.lanczos_stats()["cycle"]
        return e0.value, psi, alpha[:n], beta[:n]

    def lanczos_stats(self):
        """Breakdown of the last reorthogonalized lanczos() on this sector:
        device ms of the products and of the Gram-Schmidt sweeps, the sweeps'
        algorithmic bytes, restarts, vectors held, last cycle length."""
        pm, rm, rb = _lib.c_double(), _lib.c_double(), _lib.c_double()
        rs, nv, cy = _lib.c_int(), _lib.c_int(), _lib.c_int()
        check(lib().qcmg_lanczos_last_stats(self._h, pm, rm, rb, rs, nv, cy))
        return {"product_ms": pm.value, "reorth_ms": rm.value, "reorth_bytes": rb.value,
                "restarts": rs.value, "vectors": nv.value, "cycle": cy.value}

    def GS_energy(self):
        return self.lanczos(want_psi=False)[0]

    def states(self, GS_energy=1.0e12):
        """Lanczos ground state of this sector (Hamiltonian::states, method 'L').
        Returns ([State], updated GS_energy)."""
        if self.dim == 0:
            return [], GS_energy
        e0, psi, _, _ = self.lanczos()
        GS_energy = min(GS_energy, e0)
        out = []
        if e0 - GS_energy <= max(MIN_GAP, 0.0):
            out.append(State(self.sec, e0, psi))
        return out, GS_energy

    def lanczos_green(self, psi):
        """(a, b) of the continued-fraction Lanczos from the normalized
        psi: a host array, or a device tensor (anything with data_ptr())
        (LanczosGreen, Lanczos.hpp:156-183)."""
        cap = GLOBAL["max_iter_CF"] + 1
        a, b = np.zeros(cap), np.zeros(cap + 1)
        n = _lib.c_int()
        if hasattr(psi, "data_ptr"):
            p, flags = psi.data_ptr(), _lib.QCMG_DEVICE_PTRS
        else:
            p, flags = ptr(as_f64(psi)), 0
        check(lib().qcmg_lanczos_green(self._h, p, flags, GLOBAL["accur_continued_fraction"],
                                       GLOBAL["max_iter_CF"], n, ptr(a), ptr(b), cap))
        m = n.value
        return a[:m].copy(), b[: m + 1].copy()

    def block_lanczos(self, phi):
        """Block Lanczos of the start block phi (p, dim) (host array or device
        tensor): (A, B, W) with A, B lists of p' x p' blocks and W (p', p) the
        start block's Gram-Schmidt factor (qcmg_block_lanczos)."""
        p = int(phi.shape[0])
        M = max(int(14 * p * math.log(1.0 * self.dim)), 1) if self.dim else 1
        cap = GLOBAL["max_iter_BL"] + 1
        A, B, W = np.zeros(cap * p * p), np.zeros(cap * p * p), np.zeros(p * p)
        Mo, pa = _lib.c_int(), _lib.c_int()
        if hasattr(phi, "data_ptr"):
            src, flags = phi.data_ptr(), _lib.QCMG_DEVICE_PTRS
        else:
            phi = np.ascontiguousarray(phi, np.float64)
            src, flags = ptr(phi), 0
        check(lib().qcmg_block_lanczos(self._h, p, src, flags, M, GLOBAL["max_iter_BL"],
                                       GLOBAL["accur_deflation"], GLOBAL["accur_band_lanczos"],
                                       Mo, pa, ptr(A), ptr(B), ptr(W), cap))
        m, q = Mo.value, pa.value
        blocks = lambda X: [X[k * q * q:(k + 1) * q * q].reshape(q, q).copy() for k in range(m)]
        return blocks(A), blocks(B), W[:q * p].reshape(q, p).copy()

    def build_Q_matrix(self, phi):
        """(e, Q) with Q of shape (p, M) (Hamiltonian_base.hpp:229-254)."""
        p = len(phi)
        if self.dim == 0 or p == 0:
            return np.zeros(0), np.zeros((p, 0))
        M = int(14 * p * math.log(1.0 * self.dim))
        if M <= 1:
            M = 2
        phis = np.ascontiguousarray(np.array(phi, np.float64).reshape(p, self.dim))
        return self._band_lanczos(p, ptr(phis), M, lib().qcmg_band_lanczos)

    def build_Q_matrix_device(self, phi_dev):
        """build_Q_matrix with the start vectors in device memory: a
        contiguous (p, dim) float64 CUDA tensor (or any object with .shape
        and .data_ptr())."""
        p = int(phi_dev.shape[0])
        if self.dim == 0 or p == 0:
            return np.zeros(0), np.zeros((p, 0))
        if tuple(phi_dev.shape) != (p, self.dim):
            raise ValueError("start vectors must have shape (p, dim)")
        M = max(int(14 * p * math.log(1.0 * self.dim)), 2)
        return self._band_lanczos(p, phi_dev.data_ptr(), M, lib().qcmg_band_lanczos_device)

    def _band_lanczos(self, p, phi_ptr, M, fn):
        cap = GLOBAL["max_iter_BL"] + 2 * p + 2
        ev = np.zeros(cap)
        Q = np.zeros(p * cap)
        Mo = _lib.c_int()
        check(fn(self._h, p, phi_ptr, M, GLOBAL["max_iter_BL"], GLOBAL["accur_deflation"],
                 GLOBAL["accur_band_lanczos"], Mo, ptr(ev), ptr(Q), cap))
        m = Mo.value
        return ev[:m].copy(), Q[: p * m].reshape(p, m).copy()


def lanczos_batch(hamiltonians, want_psi=False, tol=None, max_iter=None, chunk=16,
                  raise_errors=True):
    """Lanczos ground states of several sectors at once (qcmg_lanczos_batch):
    each sector's recurrence runs from a captured CUDA graph of `chunk` steps
    with its coefficients on the device, all sectors side by side; results
    equal Hamiltonian.lanczos() on the FP64 path.  Returns a list of
    (E0, psi or None, iterations) in the order of `hamiltonians`; a sector
    that did not converge raises QcmgError, or with raise_errors=False each
    entry is (E0, psi, iterations, QcmgError or None)."""
    import ctypes
    n = len(hamiltonians)
    if n == 0:
        return []
    tol = GLOBAL["accur_lanczos"] if tol is None else tol
    max_iter = GLOBAL["max_iter_lanczos"] if max_iter is None else max_iter
    handles = (ctypes.c_void_p * n)(*[h._h.value for h in hamiltonians])
    e0 = np.zeros(n)
    nit = np.zeros(n, np.int32)
    st = np.zeros(n, np.int32)
    psis = [np.zeros(h.dim) if want_psi else None for h in hamiltonians]
    pp = (ctypes.c_void_p * n)(*[(p.ctypes.data if p is not None else None) for p in psis])
    check(lib().qcmg_lanczos_batch(n, handles, GLOBAL["seed"], tol, max_iter, chunk, ptr(e0),
                                   ptr(nit), pp, ptr(st)))
    if raise_errors:
        for k in range(n):
            check(int(st[k]))
        return [(float(e0[k]), psis[k], int(nit[k])) for k in range(n)]
    errs = [None if st[k] == 0 else QcmgError(int(st[k]), "sector %d of the batch: %s"
                                              % (k, "no convergence" if st[k] == -4
                                                 else "numerical breakdown"))
            for k in range(n)]
    return [(float(e0[k]), psis[k], int(nit[k]), errs[k]) for k in range(n)]


def apply_c(L, orb, pm, nup, ndn, x, z=1.0):
    """c_orb (pm=-1) / c^dagger_orb (pm=+1) applied to x on the GPU."""
    spin = orb >= L
    nup2, ndn2 = nup + (0 if spin else pm), ndn + (pm if spin else 0)
    if min(nup2, ndn2) < 0 or max(nup2, ndn2) > L:
        return np.zeros(0)
    n2 = math.comb(L, nup2) * math.comb(L, ndn2)
    y = np.zeros(n2)
    check(lib().qcmg_apply_c(L, orb, pm, nup, ndn, ptr(as_f64(x)), ptr(y), z, 0))
    return y


def _cuda_ready():
    """True when torch can hold device vectors for the library (the device
    path of the Green-function set-up); the host path is the fallback when
    torch has no GPU, e.g. for tests of the host logic."""
    try:
        import torch
    except ImportError:
        return False
    return torch.cuda.is_available()


def _concurrently(fn, args):
    """[fn(a) for a in args], each call in a thread of its own (the engine's
    calls release the interpreter lock and run on the handles' own streams),
    on the caller's device; the first exception is raised once all calls are
    done."""
    import torch
    from concurrent.futures import ThreadPoolExecutor
    dev = torch.cuda.current_device()

    def run(a):
        torch.cuda.set_device(dev)
        check(lib().qcmg_set_device(dev))
        return fn(a)
    with ThreadPoolExecutor(max_workers=len(args)) as ex:
        futs = [ex.submit(run, a) for a in args]
    return [f.result() for f in futs]


def apply_c_device(L, orbs, pm, nup, ndn, x_dev):
    """c_orb (pm=-1) / c^dagger_orb (pm=+1) of every orbital in orbs applied
    to the device vector x_dev, on the device: a (len(orbs), dim') CUDA
    tensor (dim' of the target sector)."""
    import torch
    spin = orbs[0] >= L
    nup2, ndn2 = nup + (0 if spin else pm), ndn + (pm if spin else 0)
    if min(nup2, ndn2) < 0 or max(nup2, ndn2) > L:
        return torch.zeros((len(orbs), 0), dtype=torch.float64, device=x_dev.device)
    n2 = math.comb(L, nup2) * math.comb(L, ndn2)
    out = torch.empty((len(orbs), n2), dtype=torch.float64, device=x_dev.device)
    for k, orb in enumerate(orbs):
        if (orb >= L) != spin:
            raise ValueError("orbitals of one call must have the same spin")
        check(lib().qcmg_apply_c(L, orb, pm, nup, ndn, x_dev.data_ptr(), out[k].data_ptr(), 1.0,
                                 _lib.QCMG_DEVICE_PTRS))
    return out


def halfbasis(L, N):
    d = _lib.c_size_t()
    check(lib().qcmg_halfbasis(L, N, None, 0, d))
    out = np.zeros(max(d.value, 1), np.uint32)
    check(lib().qcmg_halfbasis(L, N, ptr(out), d.value, d))
    return out[: d.value]


def halfbasis_rank(L, N, states):
    st = np.ascontiguousarray(states, np.uint32)
    out = np.zeros(max(len(st), 1), np.uint32)
    check(lib().qcmg_halfbasis_rank(L, N, ptr(st), len(st), ptr(out)))
    return out[: len(st)]


def green_function(e, v, z):
    """G for a list of complex frequencies; v is (L, M) complex.  Returns
    (nz, L, L) in the reference's orientation G[w][b, a] (as numpy [b, a])."""
    e = as_f64(e)
    v = np.asarray(v, np.complex128)
    L, M = v.shape
    zs = np.atleast_1d(np.asarray(z, np.complex128))
    vv = np.ascontiguousarray(v.T).view(np.float64).reshape(-1)   # column-major (a + L i)
    zz = np.ascontiguousarray(zs).view(np.float64)
    G = np.zeros(2 * L * L * len(zs))
    check(lib().qcmg_green_function(L, M, ptr(e), ptr(vv), len(zs), ptr(zz), ptr(G)))
    Gc = G.view(np.complex128).reshape(len(zs), L, L)   # [w][a][b] = G[b + a L]
    return np.transpose(Gc, (0, 2, 1)).copy()           # numpy [b, a]


def streamline(e, v, wtol=None, vtol=None):
    """Merges degenerate poles (src_ed/Q_matrix.hpp:180-223).  v is (L, M)."""
    wtol = GLOBAL["Qmatrix_wtol"] if wtol is None else wtol
    vtol = GLOBAL["Qmatrix_vtol"] if vtol is None else vtol
    L, M = v.shape
    if vtol < 1e-12:
        return e, v
    e2, cols = [], []
    i = 0
    while i < M:
        j = i + 1
        while j < M and abs(e[j] - e[i]) <= wtol:
            j += 1
        if j - i == 1:
            if np.sum(np.abs(v[:, i]) ** 2) >= vtol:
                e2.append(e[i])
                cols.append(v[:, i])
        else:
            Q = v[:, i:j]
            d, U = np.linalg.eigh(Q @ Q.conj().T)
            for k in range(L):
                if d[k] > vtol:
                    e2.append(e[i])
                    cols.append(U[:, k] * math.sqrt(d[k]))
        i = j
    if not cols:
        return np.zeros(0), np.zeros((L, 0), v.dtype)
    return np.array(e2), np.array(cols).T


class ModelInstance:
    """Instance of a cluster model with parameter values and target sectors."""

    def __init__(self, model, values, sectors, label=0):
        self.model, self.label = model, label
        self.values = {k: float(v) for k, v in values.items() if k in model.operators}
        self.target_sectors = [Sector(s) for s in sectors.split("/")]
        up, dn, _ = model.combine(self.values)
        self.mixing = 4 if (sorted(up) != sorted(dn) or any(s.S for s in self.target_sectors)) else 0
        self.gs_solved = self.gf_solved = False
        self.states = []
        self.GS_energy = None
        self.E0 = None
        self._H = {}
        self.gf_method = GLOBAL["GF_method"]
        if self.gf_method not in ("L", "F", "M"):
            raise ValueError("GF_method must be 'L' (band Lanczos), 'F' (continued fractions) "
                             "or 'M' (matrix continued fractions)")

    def hamiltonian(self, nup, ndn):
        key = (nup, ndn)
        if key not in self._H:
            self._H[key] = Hamiltonian(self.model, self.values, Sector.of(nup, ndn))
        return self._H[key]

    def gs_hamiltonians(self):
        """The Hamiltonians of the target sectors that ground_state solves
        (empty sectors left out), for solving many instances at once with
        lanczos_batch."""
        out = []
        for s in self.target_sectors:
            H = self.hamiltonian(s.nup, s.ndn)
            if H.dim:
                out.append(H)
        return out

    def ground_state(self, solved=None):
        """(GS energy, sector string) -- model_instance::low_energy_states.
        solved: optional {Hamiltonian: (E0, psi)} of the target sectors,
        computed beforehand (lanczos_batch); the sectors' Lanczos runs are then
        skipped and the states are selected as the reference does."""
        if self.gs_solved:
            return self.GS_energy, self._gs_string()
        E = 1.0e12
        states = []
        for s in self.target_sectors:
            H = self.hamiltonian(s.nup, s.ndn)
            if H.dim == 0:
                continue
            if solved is not None and H in solved:
                e0, psi = solved[H]
                E = min(E, e0)
                if e0 - E <= max(MIN_GAP, 0.0):
                    states.append(State(H.sec, e0, psi))
                continue
            st, E = H.states(E)
            states += st
        E0 = min(x.energy for x in states)
        T = GLOBAL["temperature"]
        if T < 1e-9:
            states = [x for x in states if x.energy - E0 <= SMALL_VALUE]
            for x in states:
                x.weight = 1.0 / len(states)
        else:
            w = np.array([math.exp(-(x.energy - E0) / T) for x in states])
            for x, wi in zip(states, w / w.sum()):
                x.weight = wi
        states = [x for x in states if x.weight >= GLOBAL["minimum_weight"]]
        tot = sum(x.weight for x in states)
        for x in states:
            x.weight /= tot
        if self.mixing == 0 and any(x.sec.S for x in states):
            self.mixing = 4
        self.states = states
        self.GS_energy = min(x.energy for x in states)
        self.E0 = sum(x.weight * x.energy for x in states)
        self.gs_solved = True
        return self.GS_energy, self._gs_string()

    def _gs_string(self):
        return "/".join(x.sec.name() for x in self.states)

    def _qmatrix_state(self, st, spin_down):
        L = self.model.n_orb
        ns = self.model.n_sites
        spin = 1 if spin_down else 0
        device = _cuda_ready()
        psi_dev = self._psi_device(st) if device else None

        def block(pm):
            nup2 = st.sec.nup + (0 if spin else pm)
            ndn2 = st.sec.ndn + (pm if spin else 0)
            if min(nup2, ndn2) < 0 or max(nup2, ndn2) > L:
                return None
            H = self.hamiltonian(nup2, ndn2)
            if H.dim == 0:
                return None
            if device:
                # c / c^dagger applied on the device, start vectors left there
                e, Q = H.build_Q_matrix_device(
                    apply_c_device(L, [o + spin * L for o in range(ns)], pm, st.sec.nup,
                                   st.sec.ndn, psi_dev))
            else:
                phi = [apply_c(L, o + spin * L, pm, st.sec.nup, st.sec.ndn, st.psi)
                       for o in range(ns)]
                e, Q = H.build_Q_matrix(phi)
            e = e - st.energy
            if pm == -1:
                e = -e
            e, Q = streamline(e, Q.astype(np.complex128))
            if pm == 1:
                Q = Q.conj()
            return e, Q

        # the hole and particle sectors are independent band Lanczos runs on
        # handles of their own (own streams): on the device they run at once
        res = _concurrently(block, (-1, 1)) if device else [block(pm) for pm in (-1, 1)]
        blocks = {pm: r for pm, r in zip((-1, 1), res) if r is not None}
        es = [blocks[pm][0] for pm in (-1, 1) if pm in blocks]
        vs = [blocks[pm][1] for pm in (-1, 1) if pm in blocks]
        e = np.concatenate(es) if es else np.zeros(0)
        v = np.concatenate(vs, axis=1) if vs else np.zeros((ns, 0), np.complex128)
        self._check_norm(v)
        return e, v * math.sqrt(st.weight)

    @staticmethod
    def _psi_device(st):
        """The state's vector as a device tensor, uploaded once per state."""
        import torch
        d = getattr(st, "_psi_dev", None)
        if d is None:
            d = torch.from_numpy(np.ascontiguousarray(st.psi, np.float64)).to("cuda")
            st._psi_dev = d
        return d

    @staticmethod
    def _check_norm(v):
        D = v @ v.conj().T - np.eye(v.shape[0])
        err = float(np.sum(np.abs(D) ** 2))
        if err > GLOBAL["accur_Q_matrix"]:
            raise QcmgError(-6, f"Q-matrix does not satisfy unitary condition by {err}")

    def Green_function_solve(self):
        if self.gf_solved:
            return
        self.ground_state()
        solve = {"F": self._cf_state, "M": self._mcf_state}.get(self.gf_method, self._qmatrix_state)
        for st in self.states:
            if self.mixing & 4 and self.gf_method == "L" and _cuda_ready():
                self._psi_device(st)  # uploaded once, before the two spins share it
                st.gf, st.gf_down = _concurrently(lambda sd: solve(st, sd), (False, True))
                continue
            st.gf = solve(st, False)
            if self.mixing & 4:
                st.gf_down = solve(st, True)
        self.gf_solved = True

    def write_qmatrix(self, path):
        """Saves the solved instance's Lehmann data, so that the lattice stage can
        run from the file without the impurity solve.  Per kept state and spin
        block, the Q-matrix datasets of the reference's Q_matrix::write_hdf5
        (src_ed/Q_matrix.hpp:322-332: L, M, e, v), with the state's sector,
        energy and weight, and the instance's parameter values, mixing and
        energies.  The container is a NumPy .npz archive, since no HDF5 library
        is part of this package.  Needs GF_method 'L'."""
        if self.gf_method != "L":
            raise ValueError("Q-matrix files need GF_method 'L'")
        self.Green_function_solve()
        names = sorted(self.values)
        d = {"value_names": np.array(names), "values": np.array([self.values[n] for n in names]),
             "mixing": self.mixing, "GS_energy": self.GS_energy, "E0": self.E0,
             "n_states": len(self.states)}
        for i, st in enumerate(self.states):
            d[f"s{i}_sector"] = np.array(st.sec.name())
            d[f"s{i}_energy"] = st.energy
            d[f"s{i}_weight"] = st.weight
            for tag, blk in (("up", st.gf), ("down", st.gf_down)):
                if blk is None:
                    continue
                e, v = blk
                d[f"s{i}_{tag}_L"], d[f"s{i}_{tag}_M"] = v.shape[0], len(e)
                d[f"s{i}_{tag}_e"], d[f"s{i}_{tag}_v"] = e, v
        np.savez_compressed(path, **d)

    def read_qmatrix(self, path):
        """Restores what write_qmatrix saved: the instance is then solved (ground
        state and Green function) with no device work.  The file's parameter
        values must be this instance's."""
        with np.load(path) as f:
            vals = dict(zip([str(n) for n in f["value_names"]], f["values"].tolist()))
            if vals.keys() != self.values.keys() or any(
                    abs(vals[n] - self.values[n]) > 1e-14 * max(1.0, abs(vals[n])) for n in vals):
                raise ValueError("the Q-matrix file was written for other parameter values")
            states = []
            for i in range(int(f["n_states"])):
                st = State(Sector(str(f[f"s{i}_sector"])), float(f[f"s{i}_energy"]), None)
                st.weight = float(f[f"s{i}_weight"])
                for tag in ("up", "down"):
                    if f"s{i}_{tag}_e" in f.files:
                        e, v = f[f"s{i}_{tag}_e"], f[f"s{i}_{tag}_v"]
                        if v.shape != (int(f[f"s{i}_{tag}_L"]), int(f[f"s{i}_{tag}_M"])):
                            raise ValueError("inconsistent Q-matrix block in the file")
                        setattr(st, "gf" if tag == "up" else "gf_down", (e, v))
                states.append(st)
            self.states = states
            self.mixing = int(f["mixing"])
            self.GS_energy, self.E0 = float(f["GS_energy"]), float(f["E0"])
        self.gf_method = "L"
        self.gs_solved = self.gf_solved = True

    def _cf_state(self, st, spin_down):
        """Continued fractions of one state, as model_instance<double>::build_cf
        (model_instance.cpp:35-100): for every orbital pair o2 <= o1, the
        continued-fraction Lanczos from c_o1 psi (+ c_o2 psi), normalized,
        for the electron (pm = +1) and hole (pm = -1) parts.  Returns
        {(pm, o1, o2): (a, b)} in evaluation form (continued_fraction.cpp:30-37:
        b squared with b[0] = |c psi|^2 * weight, a shifted by the energy)."""
        L, ns = self.model.n_orb, self.model.n_sites
        spin = 1 if spin_down else 0
        frac = {}
        for pm in (-1, 1):
            nup2 = st.sec.nup + (0 if spin else pm)
            ndn2 = st.sec.ndn + (pm if spin else 0)
            if min(nup2, ndn2) < 0 or max(nup2, ndn2) > L:
                continue
            H = self.hamiltonian(nup2, ndn2)
            if H.dim == 0:
                continue
            orbs = [o + spin * L for o in range(ns)]
            if _cuda_ready():
                phi = apply_c_device(L, orbs, pm, st.sec.nup, st.sec.ndn, self._psi_device(st))
            else:
                phi = np.array([apply_c(L, o, pm, st.sec.nup, st.sec.ndn, st.psi) for o in orbs])
            for o1 in range(ns):
                for o2 in range(o1 + 1):
                    x = phi[o1] + phi[o2] if o2 != o1 else phi[o1]
                    norm = float((x * x).sum())
                    if norm <= 1e-14:
                        continue
                    a, b = H.lanczos_green(x / math.sqrt(norm))
                    b = b ** 2
                    b[0] = norm * st.weight
                    a = a - st.energy if pm == 1 else st.energy - a
                    frac[(pm, o1, o2)] = (a, b)
        return frac

    def _mcf_state(self, st, spin_down):
        """Matrix continued fractions of one state, as model_instance::build_mcf
        (model_instance.hpp:847-955): per part (pm = -1 holes, +1 electrons)
        the start block c_o psi for all cluster orbitals, factored phi = q W
        with W scaled by sqrt(weight), block Lanczos on q (polar coupling
        blocks), and the diagonal blocks shifted by the energy.  Returns a
        list of (pm, A, B, W)."""
        L, ns = self.model.n_orb, self.model.n_sites
        spin = 1 if spin_down else 0
        parts = []
        for pm in (-1, 1):
            nup2 = st.sec.nup + (0 if spin else pm)
            ndn2 = st.sec.ndn + (pm if spin else 0)
            if min(nup2, ndn2) < 0 or max(nup2, ndn2) > L:
                continue
            H = self.hamiltonian(nup2, ndn2)
            if H.dim == 0:
                continue
            orbs = [o + spin * L for o in range(ns)]
            if _cuda_ready():
                phi = apply_c_device(L, orbs, pm, st.sec.nup, st.sec.ndn, self._psi_device(st))
            else:
                phi = np.array([apply_c(L, o, pm, st.sec.nup, st.sec.ndn, st.psi) for o in orbs])
            A, B, W = H.block_lanczos(phi)
            if not A:
                continue
            pa = A[0].shape[0]
            eye = np.eye(pa)
            A = [a - st.energy * eye if pm == 1 else st.energy * eye - a for a in A]
            parts.append((pm, A, B, W * math.sqrt(st.weight)))
        return parts

    @staticmethod
    def _mcf_green(parts, zs):
        """G(z) (nz, L, L) of one state's matrix continued fractions: each part
        W^T F_0(z) W with F_M = 0, F_j = (z - A_j - B_j^T F_{j+1} B_j)^-1
        (matrix_continued_fraction.hpp:139-185), the hole part transposed
        (mcf_set.hpp:112-130)."""
        G = None
        for pm, A, B, W in parts:
            pa = A[0].shape[0]
            eye = np.eye(pa)[None]
            F = np.zeros((len(zs), pa, pa), np.complex128)
            for j in range(len(A) - 1, -1, -1):
                S = B[j].T[None] @ F @ B[j][None] if j < len(A) - 1 else 0.0
                F = np.linalg.inv(zs[:, None, None] * eye - A[j][None] - S)
            g = W.T[None] @ F @ W[None]
            if pm == -1:
                g = g.transpose(0, 2, 1)
            G = g if G is None else G + g
        return G

    def _cf_green(self, frac, zs):
        """G(z) (nz, L, L) of one state's continued fractions
        (continued_fraction_set::Green_function, real case,
        continued_fraction_set.cpp:63-98): diagonal elements from the
        (o, o) fractions, off-diagonal ones 0.5 (G_{o1+o2} - G_o1o1 - G_o2o2)."""
        ns = self.model.n_sites
        keys = list(frac)
        nmax = max((len(frac[k][0]) for k in keys), default=0)
        # all fractions at once, padded with b = 0 (a zero term leaves G as it is)
        A = np.zeros((len(keys), nmax))
        B = np.zeros((len(keys), nmax))
        for i, k in enumerate(keys):
            a, b = frac[k]
            A[i, :len(a)] = a
            B[i, :len(a)] = b[:len(a)]
        val = np.zeros((len(keys), len(zs)), np.complex128)
        for j in range(nmax - 1, -1, -1):
            val = B[:, j, None] / (zs[None, :] - A[:, j, None] - val)
        part = {}
        for i, (pm, o1, o2) in enumerate(keys):
            part[(o1, o2)] = part.get((o1, o2), 0.0) + val[i]
        G = np.zeros((len(zs), ns, ns), np.complex128)
        zero = np.zeros(len(zs), np.complex128)
        d = [part.get((o, o), zero) for o in range(ns)]
        for o in range(ns):
            G[:, o, o] = d[o]
        for o1 in range(ns):
            for o2 in range(o1):
                t = 0.5 * (part.get((o1, o2), zero) - d[o1] - d[o2])
                G[:, o1, o2] = t
                G[:, o2, o1] = t
        return G

    def qmatrix(self, spin_down=False):
        """(e, v) of the first state, v of shape (L, M)."""
        if self.gf_method != "L":
            raise ValueError("the Q-matrix exists with GF_method 'L' only")
        self.Green_function_solve()
        st = self.states[0]
        return st.gf_down if (spin_down and self.mixing & 4) else st.gf

    def Green_function(self, z, spin_down=False):
        """G(z) (n_sites x n_sites); z scalar or array (then (nz, L, L))."""
        self.Green_function_solve()
        zs = np.atleast_1d(np.asarray(z, np.complex128))
        G = None
        for st in self.states:
            gf = st.gf_down if (spin_down and self.mixing & 4) else st.gf
            if self.gf_method == "F":
                g = self._cf_green(gf, zs)
            elif self.gf_method == "M":
                g = self._mcf_green(gf, zs)
            else:
                g = green_function(*gf, zs)
            G = g if G is None else G + g
        return G[0] if np.ndim(z) == 0 else G

    def hopping_blocks(self, spin_down=False):
        """(tc, tcb, tb) with the bath diagonalized (model_instance.hpp:425-475)."""
        ns = self.model.n_sites
        T = self.model.one_body_matrix(self.values, spin_down and bool(self.mixing & 4))
        tc, tcb, tb = T[:ns, :ns], T[:ns, ns:], T[ns:, ns:]
        if tb.size and np.count_nonzero(tb - np.diag(np.diag(tb))):
            d, S = np.linalg.eigh(tb)
            tb, tcb = np.diag(d), tcb @ S
        return tc, tcb, tb

    def hybridization_function(self, z, spin_down=False):
        _, tcb, tb = self.hopping_blocks(spin_down)
        ns = self.model.n_sites
        G = np.zeros((ns, ns), np.complex128)
        for i in range(tb.shape[0]):
            G += np.outer(tcb[:, i], tcb[:, i].conj()) / (z - tb[i, i])
        return G

    def self_energy(self, z, spin_down=False):
        if self.gf_method == "L":
            return self.self_energy_device([z], spin_down)[0]
        G = self.Green_function(z, spin_down)
        tc, _, _ = self.hopping_blocks(spin_down)
        S = np.linalg.inv(G) + tc
        if self.model.n_bath:
            S = S + self.hybridization_function(z, spin_down)
        return z * np.eye(len(tc)) - S

    def hybridization_function_many(self, zs, spin_down=False):
        """Gamma(z) for every z of zs at once: (nz, L, L)."""
        _, tcb, tb = self.hopping_blocks(spin_down)
        zs = np.atleast_1d(np.asarray(zs, np.complex128))
        d = np.diag(tb) if tb.size else np.zeros(0)
        w = 1.0 / (zs[:, None] - d[None, :])
        return np.einsum("ik,zk,jk->zij", tcb, w, tcb.conj())

    def self_energy_device(self, zs, spin_down=False, want_gamma=False):
        """Sigma(z) (and Gamma(z) with want_gamma) for every z of zs in one
        device call (qcmg_self_energy): the Q-matrices of the kept states, the
        batched G(z), its inverse per frequency and the bath's Gamma(z) all on
        the device.  GF_method 'L' only (the Q-matrix form)."""
        if self.gf_method != "L":
            raise ValueError("the device self-energy takes the Q-matrix (GF_method 'L')")
        self.Green_function_solve()
        zs = np.atleast_1d(np.asarray(zs, np.complex128))
        es, vs = [], []
        for st in self.states:
            e, v = st.gf_down if (spin_down and self.mixing & 4) else st.gf
            es.append(e)
            vs.append(v)
        e = np.ascontiguousarray(np.concatenate(es), np.float64)
        v = np.concatenate(vs, axis=1)
        L, M = v.shape
        tc, tcb, tb = self.hopping_blocks(spin_down)
        nb = tb.shape[0]
        vv = np.ascontiguousarray(v.T.astype(np.complex128)).view(np.float64).reshape(-1)
        cb = np.ascontiguousarray(np.asarray(tcb, np.complex128).T).view(np.float64).reshape(-1)
        eb = np.ascontiguousarray(np.diag(tb).real if nb else np.zeros(0))
        tcc = np.ascontiguousarray(np.asarray(tc, np.complex128)).view(np.float64).reshape(-1)
        zz = np.ascontiguousarray(zs).view(np.float64)
        S = np.zeros(2 * L * L * len(zs))
        Gm = np.zeros_like(S) if want_gamma else None
        check(lib().qcmg_self_energy(L, M, ptr(e) if M else None, ptr(vv) if M else None, nb,
                                     ptr(cb) if nb else None, ptr(eb) if nb else None, ptr(tcc),
                                     len(zs), ptr(zz), ptr(S), ptr(Gm)))
        S = S.view(np.complex128).reshape(len(zs), L, L)
        if want_gamma:
            return S, Gm.view(np.complex128).reshape(len(zs), L, L)
        return S

    def self_energy_many(self, zs, spin_down=False):
        """Sigma(z) for every z of zs at once: on the device for the Q-matrix
        form (self_energy_device), else one batched Green-function evaluation
        and one batched inverse on the host."""
        zs = np.atleast_1d(np.asarray(zs, np.complex128))
        if self.gf_method == "L":
            return self.self_energy_device(zs, spin_down)
        G = self.Green_function(zs, spin_down)
        if G.ndim == 2:
            G = G[None]
        tc, _, _ = self.hopping_blocks(spin_down)
        S = np.linalg.inv(G) + tc[None]
        if self.model.n_bath:
            S = S + self.hybridization_function_many(zs, spin_down)
        return zs[:, None, None] * np.eye(len(tc))[None] - S

    def tr_sigma_inf(self):
        """Trace of the self-energy's infinite-frequency limit
        (model_instance::tr_sigma_inf, src_ed/model_instance.hpp:1279-1311):
        Re Tr Sigma(i/x) at x = 1e-5, 2e-5 and 3e-5, summed over the spin
        blocks (twice the one block when both spins share it), and the
        quadratic through those three points evaluated at x = 0 (the
        reference's Neville scheme; the same polynomial in Lagrange form)."""
        x = np.array([1e-5, 2e-5, 3e-5])
        zs = 1j / x
        S = np.zeros(len(x))
        for sd in ((False, True) if self.mixing & 4 else (False,)):
            S += np.trace(self.self_energy_many(zs, sd), axis1=1, axis2=2).real
        if not self.mixing & 4:
            S *= 2.0
        lag = [np.prod([-x[j] / (x[i] - x[j]) for j in range(len(x)) if j != i])
               for i in range(len(x))]
        return float(np.dot(lag, S))

    def SEF_bath(self):
        sef = 0.0
        for sd in ((False, True) if self.mixing & 4 else (False,)):
            _, _, tb = self.hopping_blocks(sd)
            sef -= sum(x for x in np.diag(tb) if x < 0)
        return sef if self.mixing & 4 else 2.0 * sef

    def Potthoff_functional(self):
        """Cluster part E0 + SEF_bath (src_ed/qcm_ED.cpp:330-334)."""
        self.Green_function_solve()
        return self.E0 + self.SEF_bath()
