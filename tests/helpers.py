"""Shared helpers for the parity tests: build the golden models for the
engine (pyqcm_gb300) and for the CPU oracle from the same definitions."""
import numpy as np

from models import CASES, hubbard_cluster


def case_model(tag):
    nx, ny, nb, af, params, sec, gf = CASES[tag]
    ns, nb, ops = hubbard_cluster(nx, ny, nb, af)
    return ns, nb, ops, params, sec


def engine_model(tag):
    import pyqcm_gb300 as pg
    ns, nb, ops, params, sec = case_model(tag)
    m = pg.ClusterModel(ns, nb)
    for name, (typ, els) in ops.items():
        m.new_operator(name, typ, els)
    return m, params, sec


def oracle_sector(tag, sector=None):
    import qcm_oracle as qo
    ns, nb, ops, params, sec = case_model(tag)
    sec = sector or sec
    parts = dict((p[0], int(p[1:])) for p in sec.split(":"))
    N, S = parts["N"], parts["S"]
    nup, ndn = (N + S) // 2, (N - S) // 2
    up, dn, pr = qo.combine_terms(ops, params, ns + nb)
    return qo.Sector(ns + nb, nup, ndn, up, dn, pr), (up, dn, pr)


def halfop_dense_from_ref(g, prefix, op_names, params, dim):
    """Dense half-operator (hopping part + diagonal) assembled from the
    reference's HS_half_operator tables (lower triangle grouped by value)
    with the coefficients of the value map."""
    T = np.zeros((dim, dim))
    for name in op_names:
        key = f"{prefix}_{name}"
        if key + "_IJ" not in g:
            continue
        coef = params[name.rsplit("_", 1)[0]] if False else params[name.split("_")[0]]
        IJ = g[key + "_IJ"].reshape(-1, 2)
        for (I, J), v in zip(IJ, g[key + "_val"]):
            T[I, J] += coef * v
            T[J, I] += coef * v
        for r, v in zip(g[key + "_diag_r"], g[key + "_diag_v"]):
            T[r, r] += coef * v
    return T


def csr_dense(rp, col, val, diag):
    dim = len(rp) - 1
    T = np.zeros((dim, dim))
    for i in range(dim):
        for k in range(rp[i], rp[i + 1]):
            T[i, col[k]] += val[k]
        T[i, i] += diag[i]
    return T
