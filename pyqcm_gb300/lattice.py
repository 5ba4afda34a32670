"""Lattice layer (CPT / VCA / CDMFT) on the GPU engine.

Mirrors, for a lattice built from one cluster of a one-band model, the part
of pyqcm's lattice interface that feeds the k x omega integrals:
  LatticeModel      ~ pyqcm.lattice_model + QCM::new_lattice_model
                      (hopping_operator, interaction_operator, density_wave,
                      set_target_sectors, set_parameters)
  LatticeInstance   ~ lattice_model_instance (src_qcm/lattice_model_instance.cpp):
                      Potthoff_functional on a fixed (k, omega) grid,
                      periodized_Green_function / spectral_function (CPT),
                      dos, averages and potential_energy on the fixed grids,
                      CDMFT_host, CDMFT_distance
Wavevectors passed by the user are in units of 2 pi / a of the physical
lattice (the reference's physdual basis); internally K = S k with S the
superlattice, so that phases are exp(2 pi i K.R) for superlattice
translations R in the superlattice basis (src_qcm/CPT.cpp:27-31).
"""
import itertools
import math

import numpy as np

from . import _lib
from ._lib import as_f64, check, lib, ptr
from .ed import ClusterModel, ModelInstance

GRID = {"k": None, "w": None, "wt": None}


def set_wavevector_grid(nkx, nky=1, nkz=1):
    """k grid of the fixed-grid integrals (QCM::set_wavevector_grid)."""
    GRID["k"] = (int(nkx), int(nky), int(nkz))


def discrete_integration_grid(freqs, weights):
    """Imaginary-frequency grid and weights (pyqcm.discrete_integration_grid)."""
    GRID["w"] = np.asarray(freqs, np.float64).copy()
    GRID["wt"] = np.asarray(weights, np.float64).copy()


def legendre_frequency_grid(w1, w2, n1, n2, n3):
    """Gauss-Legendre grid on [0,w1], [w1,w2] and [w2, inf) (1/w mapped),
    weights including 1/pi, as pyqcm.legendre_frequency_grid builds it
    (pyqcm/__init__.py:3040-3066)."""
    w = np.zeros(n1 + n2 + n3)
    p = np.zeros(n1 + n2 + n3)
    x, a = np.polynomial.legendre.leggauss(n1)
    w[:n1] = w1 * 0.5 * (x + 1)
    p[:n1] = a * w1 * 0.5
    x, a = np.polynomial.legendre.leggauss(n2)
    w[n1:n1 + n2] = w1 + 0.5 * (w2 - w1) * (x + 1)
    p[n1:n1 + n2] = a * (w2 - w1) * 0.5
    x, a = np.polynomial.legendre.leggauss(n3)
    w[n1 + n2:] = 1.0 / ((1.0 / w2) * 0.5 * np.flip(x + 1))
    p[n1 + n2:] = np.flip(a) * (1.0 / w2) * 0.5 * w[n1 + n2:] ** 2
    return w, p / np.pi


class _Op:
    def __init__(self, name, kind):
        self.name, self.kind = name, kind
        self.intra = []   # (r, c, v) spin-orbital elements inside the cluster
        self.inter = []   # (r, c, R tuple, v) spin-orbital elements to other clusters


class LatticeModel:
    """Lattice of identical clusters (one band, one cluster per unit).

    cluster: ClusterModel (its n_sites cluster orbitals are the sites below;
    bath orbitals, if any, come after them); sites: integer positions of the
    cluster sites; superlattice: the dim integer superlattice vectors."""

    def __init__(self, cluster, sites, superlattice, name="lattice"):
        self.cluster = cluster
        self.name = name
        self.sites = [tuple(int(c) for c in s) + (0,) * (3 - len(s)) for s in sites]
        assert len(self.sites) == cluster.n_sites
        self.dim = len(superlattice)
        S = np.zeros((3, 3))
        for i, v in enumerate(superlattice):
            S[i, :len(v)] = v
        for i in range(self.dim, 3):  # pad unused dimensions with unit vectors
            S[i, i] = 1.0
        self.S = S
        self.Sinv = np.linalg.inv(S.T)  # fractional coordinates: x = Sinv r
        self.site_index = {s: i for i, s in enumerate(self.sites)}
        self.ops = {}
        self.target_sectors = None
        self.params = {}
        # the chemical potential is always present, -1 per site and spin
        # (lattice_model::add_chemical_potential, src_qcm/lattice_model.cpp:286-295)
        mu = self._op("mu", "one-body")
        no = cluster.n_orb
        for i in range(len(self.sites)):
            mu.intra += [(i, i, -1.0), (i + no, i + no, -1.0)]

    # -- geometry
    def _fold(self, r):
        """(site index, superlattice translation n) with r = site + n.S."""
        rng = range(-3, 4)
        for n in itertools.product(rng, repeat=self.dim):
            nn = list(n) + [0] * (3 - self.dim)
            base = tuple(int(round(r[i] - sum(nn[k] * self.S[k, i] for k in range(3)))) for i in range(3))
            if base in self.site_index:
                return self.site_index[base], tuple(nn)
        raise ValueError(f"position {r} is not on the lattice")

    def _op(self, name, kind):
        if name not in self.ops:
            self.ops[name] = _Op(name, kind)
        return self.ops[name]

    # -- operators (QCM::hopping_operator / interaction_operator / density_wave)
    def hopping_operator(self, name, link, amplitude, tau=1, sigma=0):
        """One-body operator along `link` (tau=1: real hopping c+_i c_j + h.c.;
        link (0,0,0) with tau=0: on-site term); sigma=0 spin independent,
        sigma=3: spin-dependent sign (+ up, - down)."""
        link = tuple(int(c) for c in link) + (0,) * (3 - len(link))
        op = self._op(name, "one-body")
        no = self.cluster.n_orb
        spins = ((0, 1.0), (1, 1.0)) if sigma == 0 else ((0, 1.0), (1, -1.0))
        for i, s in enumerate(self.sites):
            tgt = tuple(s[k] + link[k] for k in range(3))
            j, n = self._fold(tgt)
            for spin, sgn in spins:
                a = amplitude * sgn
                ri, rj = i + spin * no, j + spin * no
                if link == (0, 0, 0):
                    op.intra.append((ri, ri, a))
                elif n == (0, 0, 0):
                    op.intra.append((min(ri, rj), max(ri, rj), a))
                else:
                    op.inter.append((ri, rj, n, a))
                    op.inter.append((rj, ri, tuple(-c for c in n), np.conj(a)))

    def interaction_operator(self, name, amplitude=1.0, type="Hubbard"):
        if type != "Hubbard":
            raise ValueError("only the on-site Hubbard interaction factorizes")
        op = self._op(name, "interaction")
        no = self.cluster.n_orb
        for i in range(len(self.sites)):
            op.intra.append((i, i + no, amplitude))

    def density_wave(self, name, type, Q, amplitude=1.0, phase=0.0):
        """Site density wave with wavevector Q (units of pi): 'Z' spin density
        (+ up, - down) or 'N' charge density, amplitude cos(pi Q.r + phase)."""
        Q = tuple(Q) + (0,) * (3 - len(Q))
        op = self._op(name, "one-body")
        no = self.cluster.n_orb
        for i, s in enumerate(self.sites):
            c = math.cos(math.pi * sum(Q[k] * s[k] for k in range(3)) + math.pi * phase)
            c = 0.0 if abs(c) < 1e-14 else c
            if type == "Z":
                op.intra += [(i, i, amplitude * c), (i + no, i + no, -amplitude * c)]
            elif type in ("N", "cdw"):
                op.intra += [(i, i, amplitude * c), (i + no, i + no, amplitude * c)]
            else:
                raise ValueError(f"density wave type {type} does not factorize")

    def finalize(self):
        """Registers the cluster part of every lattice operator in the ED model."""
        for name, op in self.ops.items():
            if name not in self.cluster.operators and op.intra:
                self.cluster.new_operator(name, op.kind, op.intra)

    def set_target_sectors(self, sectors):
        self.target_sectors = sectors if isinstance(sectors, str) else "/".join(sectors)

    def set_parameters(self, values):
        """values: {name: value}; cluster values are 'name_1' and default to the
        lattice value (parameter_set implicit equivalences,
        src_qcm/parameter_set.cpp:103-124)."""
        self.params = dict(values)

    def cluster_values(self):
        v = {}
        for name in set(self.ops) | set(self.cluster.operators):
            if name + "_1" in self.params:
                v[name] = self.params[name + "_1"]
            elif name in self.params:
                v[name] = self.params[name]
        return v

    def lattice_values(self):
        return {name: self.params.get(name, 0.0) for name in self.ops}

    # -- Fourier data of t(k) - t_c
    def fourier(self, spin_down):
        L = self.cluster.n_sites
        no = self.cluster.n_orb
        off = no if spin_down else 0
        lv, cv = self.lattice_values(), self.cluster_values()
        hdiff = np.zeros((L, L), np.complex128)
        R = [(0, 0, 0)]
        els = []
        for name, op in self.ops.items():
            if op.kind != "one-body":
                continue
            pl, pc = lv.get(name, 0.0), cv.get(name, 0.0)
            for r, c, v in op.intra:
                if off <= r < off + L and off <= c < off + L:
                    hdiff[r - off, c - off] += (pl - pc) * v
                    if r != c:
                        hdiff[c - off, r - off] += (pl - pc) * np.conj(v)
            for r, c, n, v in op.inter:
                if off <= r < off + L and off <= c < off + L and pl != 0.0:
                    if n not in R:
                        R.append(n)
                    els.append((r - off, c - off, R.index(n), pl * v))
        gpos = np.array([self.Sinv @ np.array(s, float) for s in self.sites])
        return np.array(R, np.float64), els, hdiff, gpos

    def instance(self, label=0):
        return LatticeInstance(self, label)


class _LatticeBlock:
    """qcmg_lattice handle of one spin block."""

    def __init__(self, model, spin_down):
        R, els, hdiff, gpos = model.fourier(spin_down)
        L = model.cluster.n_sites
        er = np.array([e[0] for e in els], np.int32)
        ec = np.array([e[1] for e in els], np.int32)
        en = np.array([e[2] for e in els], np.int32)
        ev = np.ascontiguousarray(np.array([e[3] for e in els], np.complex128)).view(np.float64)
        hd = np.ascontiguousarray(hdiff).view(np.float64).reshape(-1)
        h = _lib.vp()
        check(lib().qcmg_lattice_create(L, len(R), ptr(np.ascontiguousarray(R)), len(els),
                                        ptr(er), ptr(ec), ptr(en), ptr(ev), ptr(hd),
                                        ptr(np.ascontiguousarray(gpos)), h))
        self._h = h
        self.hdiff = hdiff
        self.L = L

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.qcmg_lattice_destroy(h)

    def set_green(self, e, v, tcb, tb):
        L = self.L
        vv = np.ascontiguousarray(np.asarray(v, np.complex128).T).view(np.float64).reshape(-1)
        tc = np.ascontiguousarray(np.asarray(tcb, np.complex128).T).view(np.float64).reshape(-1)
        eb = np.ascontiguousarray(np.diag(tb).real if np.size(tb) else np.zeros(0))
        check(lib().qcmg_lattice_set_green(self._h, len(e), ptr(as_f64(e)),
                                           ptr(vv) if len(e) else None, len(eb),
                                           ptr(tc) if len(eb) else None,
                                           ptr(as_f64(eb)) if len(eb) else None))


class LatticeInstance:
    def __init__(self, model, label=0):
        model.finalize()
        self.model = model
        self.label = label
        self.cluster = ModelInstance(model.cluster, model.cluster_values(), model.target_sectors,
                                     label)
        self._blocks = None

    @property
    def mixing(self):
        self.cluster.ground_state()
        up, dn, _ = self.model.cluster.combine(self.cluster.values)
        lv = self.model.lattice_values()
        return self.cluster.mixing

    def _spin_blocks(self):
        self.cluster.Green_function_solve()
        if self._blocks is None:
            spins = (False, True) if self.cluster.mixing & 4 else (False,)
            self._blocks = {}
            for sd in spins:
                blk = _LatticeBlock(self.model, sd)
                e, v = self.cluster.qmatrix(sd)
                # all kept states contribute: concatenate their Q-matrices
                es, vs = [], []
                for st in self.cluster.states:
                    ee, vv = st.gf_down if (sd and self.cluster.mixing & 4) else st.gf
                    es.append(ee)
                    vs.append(vv)
                _, tcb, tb = self.cluster.hopping_blocks(sd)
                blk.set_green(np.concatenate(es), np.concatenate(vs, axis=1), tcb, tb)
                self._blocks[sd] = blk
        return self._blocks

    def ground_state(self):
        return self.cluster.ground_state()

    def Potthoff_functional(self):
        """Omega per site on the fixed grid (lattice_model_instance.cpp:503-584)."""
        if GRID["w"] is None or GRID["k"] is None:
            raise ValueError("set the k grid and the discrete frequency grid first")
        blocks = self._spin_blocks()
        nkx, nky, nkz = GRID["k"]
        dims = (nkx, nky if self.model.dim >= 2 else 1, nkz if self.model.dim >= 3 else 1)
        Iv = 0.0
        for sd, blk in blocks.items():
            out = _lib.c_double()
            check(lib().qcmg_sef_grid(blk._h, len(GRID["w"]), ptr(GRID["w"]), ptr(GRID["wt"]),
                                      dims[0], dims[1], dims[2], out))
            Iv += out.value
        up_down = bool(self.cluster.mixing & 4)
        if not up_down:
            Iv *= 2.0
        omega_trace = -Iv
        diag = 0.0
        for sd, blk in blocks.items():
            diag -= float(np.real(np.trace(blk.hdiff)))
        if not up_down:
            diag *= 2.0
        omega_diag = 0.5 * diag
        omega_clus = self.cluster.Potthoff_functional()
        return (omega_trace - omega_diag + omega_clus) / len(self.model.sites)

    def _K(self, k):
        k = np.atleast_2d(np.asarray(k, np.float64))
        k3 = np.zeros((len(k), 3))
        k3[:, :k.shape[1]] = k
        return np.ascontiguousarray(k3 @ self.model.S.T)

    def periodized_Green_function(self, z, k, spin_down=False):
        """g(k, z) for complex frequencies z (array) and wavevectors k (nk x 3,
        units of 2 pi): returns (nz, nk) complex (one band)."""
        blk = self._spin_blocks()[bool(spin_down) and bool(self.cluster.mixing & 4)]
        zs = np.ascontiguousarray(np.atleast_1d(np.asarray(z, np.complex128)))
        K = self._K(k)
        g = np.zeros(2 * len(zs) * len(K))
        check(lib().qcmg_cpt_periodized(blk._h, len(zs), ptr(zs.view(np.float64)), len(K), ptr(K),
                                        ptr(g)))
        return g.view(np.complex128).reshape(len(zs), len(K))

    def spectral_function(self, w, k, eta=0.1, spin_down=False):
        """A(k, w) = -Im g(k, w + i eta) (pyqcm/_spectral.py:374-392): (nw, nk)."""
        z = np.asarray(w, np.float64) + 1j * eta
        return -self.periodized_Green_function(z, k, spin_down).imag

    def dos(self, z):
        """Density of states at complex frequency z on the wavevector grid
        (lattice_model_instance::dos with use_grid, src_qcm/average.cpp:
        294-347): [D_up, D_down], D = -(1/pi) Im Tr mean_K Gcpt(K, z) / L for
        the one band of these models; z may be an array (then (nz, 2))."""
        if GRID["k"] is None:
            raise ValueError("set the wavevector grid first (set_wavevector_grid)")
        nkx, nky, nkz = GRID["k"]
        dims = (nkx, nky if self.model.dim >= 2 else 1, nkz if self.model.dim >= 3 else 1)
        zs = np.atleast_1d(np.asarray(z, np.complex128))
        zz = np.ascontiguousarray(zs).view(np.float64)
        blocks = self._spin_blocks()
        D = np.zeros((len(zs), 2))
        for sd, blk in blocks.items():
            L = blk.L
            out = np.zeros(2 * len(zs) * L * L)
            check(lib().qcmg_lattice_kmean(blk._h, len(zs), ptr(zz), dims[0], dims[1], dims[2], 0.0,
                                           ptr(out)))
            g = out.view(np.complex128).reshape(len(zs), L, L)
            d = -np.trace(g, axis1=1, axis2=2).imag / np.pi / L
            D[:, 1 if sd else 0] = d
        if not self.cluster.mixing & 4:  # normal mixing: the down part equals the up part
            D[:, 1] = D[:, 0]
        return D[0] if np.ndim(z) == 0 else D

    def averages(self, ops=None):
        """Lattice averages of one-body operators on the frequency and wavevector
        grids (lattice_model_instance::averages with grid_freqs,
        src_qcm/average.cpp:24-105; integrand average_integrand_k, 157-190):

            <O> = norm sum_w wt_w mean_K Re sum_e v_e [Gcpt(K, i w) - G_pole]_(c_e, r_e) phase_n(e)(K)

        with G_pole = 1/(i w - 2) on the diagonal, the spin-up elements counted
        twice when both spins share one block, and norm = 1/n_sites (mu:
        -1/n_sites, lattice_model.cpp:383-385).  The device returns, per
        frequency, the K means of Gcpt times each translation's phase; each
        operator is a linear form in those blocks.  ops: names (interactions
        are skipped, as in the reference); default every one-body operator.
        Returns {name: value}."""
        if GRID["w"] is None or GRID["k"] is None:
            raise ValueError("set the k grid and the discrete frequency grid first")
        names = [n for n, op in self.model.ops.items() if op.kind == "one-body"] if ops is None \
            else [n for n in ops if self.model.ops[n].kind == "one-body"]
        blocks = self._spin_blocks()
        up_down = bool(self.cluster.mixing & 4)
        L, no = self.model.cluster.n_sites, self.model.cluster.n_orb
        nkx, nky, nkz = GRID["k"]
        dims = (nkx, nky if self.model.dim >= 2 else 1, nkz if self.model.dim >= 3 else 1)
        w, wt = GRID["w"], GRID["wt"]
        zs = np.ascontiguousarray(1j * w)
        gpole = 1.0 / (zs - 2.0)
        # the K grid as the device lays it out, for the mean phase of the G_pole term
        ax = [(np.arange(g) / g) if g > 1 else np.zeros(1) for g in dims]
        Kg = np.stack(np.meshgrid(*ax, indexing="ij"), -1).reshape(-1, 3)
        I = dict.fromkeys(names, 0.0)
        for sd, blk in blocks.items():
            off = no if sd else 0
            inb = lambda a, b: off <= a < off + L and off <= b < off + L
            elems, Rs = {}, [(0, 0, 0)]
            for name in names:
                op, lst = self.model.ops[name], []
                for r, c, v in op.intra:  # the cluster's (r, c) and its conjugate (c, r)
                    for a, b, x in [(r, c, v)] + ([(c, r, np.conj(v))] if r != c else []):
                        if inb(a, b):
                            lst.append((a - off, b - off, 0, x))
                for r, c, n, v in op.inter:
                    if inb(r, c):
                        if n not in Rs:
                            Rs.append(n)
                        lst.append((r - off, c - off, Rs.index(n), v))
                elems[name] = lst
            R = np.array(Rs, np.float64)
            mom = np.zeros((len(zs), len(Rs), L, L), np.complex128)
            for m0 in range(0, len(Rs), 16):
                Rc = np.ascontiguousarray(R[m0:m0 + 16])
                out = np.zeros(2 * len(zs) * len(Rc) * L * L)
                check(lib().qcmg_lattice_kmoments(blk._h, len(zs), ptr(zs.view(np.float64)),
                                                  dims[0], dims[1], dims[2], 0.0, len(Rc), ptr(Rc),
                                                  ptr(out)))
                mom[:, m0:m0 + len(Rc)] = out.view(np.complex128).reshape(len(zs), len(Rc), L, L)
            phm = np.exp(2j * np.pi * (Kg @ R.T)).mean(axis=0)
            for name, lst in elems.items():
                z = np.zeros(len(zs), np.complex128)
                for r, c, m, v in lst:
                    z += v * mom[:, m, c, r]
                    if r == c:
                        z -= v * gpole * phm[m]
                I[name] += float(np.sum(wt * z.real))
        norm = 1.0 / len(self.model.sites)
        return {n: (2.0 if not up_down else 1.0) * I[n] * (-norm if n == "mu" else norm)
                for n in names}

    def potential_energy(self):
        """Potential energy per site on the frequency and wavevector grids
        (lattice_model_instance::potential_energy with grid_freqs,
        src_qcm/average.cpp:530-584; integrand potential_energy_integrand_k,
        669-686):

            E_pot = (1/2L) sum_w wt_w Re[ s Tr(Sigma(i w) mean_K Gcpt(K, i w)) - tr_sigma_inf/(i w - 2) ]

        with s = 2 when both spins share one block (else the blocks are
        summed).  Sigma does not depend on K, so the K sum is the device's K
        mean of Gcpt, the same one as the density of states."""
        if GRID["w"] is None or GRID["k"] is None:
            raise ValueError("set the k grid and the discrete frequency grid first")
        blocks = self._spin_blocks()
        up_down = bool(self.cluster.mixing & 4)
        nkx, nky, nkz = GRID["k"]
        dims = (nkx, nky if self.model.dim >= 2 else 1, nkz if self.model.dim >= 3 else 1)
        w, wt = GRID["w"], GRID["wt"]
        zs = np.ascontiguousarray(1j * w)
        tr = np.zeros(len(zs), np.complex128)
        for sd, blk in blocks.items():
            L = blk.L
            out = np.zeros(2 * len(zs) * L * L)
            check(lib().qcmg_lattice_kmean(blk._h, len(zs), ptr(zs.view(np.float64)), dims[0],
                                           dims[1], dims[2], 0.0, ptr(out)))
            g = out.view(np.complex128).reshape(len(zs), L, L)
            S = self.cluster.self_energy_many(zs, sd)
            tr += np.einsum("wij,wji->w", S, g)
        if not up_down:
            tr *= 2.0
        e = tr - self.cluster.tr_sigma_inf() / (zs - 2.0)
        return 0.5 * float(np.sum(wt * e.real)) / len(self.model.sites)

    def projected_Green_function(self, w, kside, spin_down=False):
        blk = self._spin_blocks()[bool(spin_down) and bool(self.cluster.mixing & 4)]
        w = as_f64(w)
        L = blk.L
        out = np.zeros(2 * len(w) * L * L)
        check(lib().qcmg_cdmft_projected(blk._h, len(w), ptr(w), kside, self.model.dim, ptr(out)))
        return out.view(np.complex128).reshape(len(w), L, L)

    def CDMFT_host(self, freqs, weights, kside=32):
        """G_host(i w) = PGF^-1 + Sigma_c + t_c - i w (src_qcm/CPT.cpp:356-424)."""
        self._host_freqs = as_f64(freqs)
        self._host_weights = as_f64(weights)
        self._host = {}
        spins = (False, True) if self.cluster.mixing & 4 else (False,)
        zs = 1j * self._host_freqs
        for sd in spins:
            P = self.projected_Green_function(self._host_freqs, kside, sd)
            tc, _, _ = self.cluster.hopping_blocks(sd)
            X = self.cluster.self_energy_many(zs, sd)
            eye = np.eye(len(tc))
            self._host[sd] = np.linalg.inv(P) + X + tc[None] - zs[:, None, None] * eye[None]
        return self._host

    def CDMFT_distance(self, bath_values):
        """sum_w w_n |Gamma(i w; p) + G_host(i w)|^2 dw / dim^2, x2 for normal
        mixing (src_qcm/CPT.cpp:519-555).  bath_values: {param: value}, named
        as the lattice model names cluster parameters ('eb1_1' is eb1 of
        cluster 1), the bare cluster name also accepted."""
        vals = dict(self.cluster.values)
        for name, x in bath_values.items():
            vals[name[:-2] if name.endswith("_1") else name] = float(x)
        inst = ModelInstance(self.model.cluster, vals, self.model.target_sectors)
        inst.mixing = self.cluster.mixing
        w = self._host_freqs
        dw = w[1] - w[0]
        dist = 0.0
        dim = None
        for sd, H in self._host.items():
            for i, wi in enumerate(w):
                g = inst.hybridization_function(1j * wi, sd) + H[i]
                dim = g.shape[0]
                dist += float(np.sum(np.abs(g) ** 2)) * self._host_weights[i]
        if self.cluster.mixing == 0:
            dist *= 2
        return dist * dw / (dim * dim)
