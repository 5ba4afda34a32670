"""Cluster models used by the golden fixtures and the parity tests.

Each model is a list of named operators given by spin-orbital matrix
elements in pyqcm's cluster convention: orbitals 0..n_orb-1 are spin up,
n_orb..2*n_orb-1 spin down; one-body elements (r, c, v) with r <= c are
completed by their Hermitian conjugate (src_ed/Operators/one_body_operator.hpp:62-71);
interaction elements (r, c, v) add v*n_r*n_c
(src_ed/Operators/interaction_operator.hpp:40-52).
"""


def _bonds_2d(nx, ny):
    """Nearest-neighbour and diagonal bonds of an open nx-by-ny cluster,
    sites numbered row-major (x fastest)."""
    nn, diag = [], []
    for y in range(ny):
        for x in range(nx):
            i = x + nx * y
            if x + 1 < nx:
                nn.append((i, i + 1))
            if y + 1 < ny:
                nn.append((i, i + nx))
            if x + 1 < nx and y + 1 < ny:
                diag.append((i, i + 1 + nx))
            if x - 1 >= 0 and y + 1 < ny:
                diag.append((i, i - 1 + nx))
    return nn, diag


def hubbard_cluster(nx, ny, n_bath=0, af=False):
    """Operators of a Hubbard cluster: t (nearest neighbour, amplitude -1),
    tp (diagonal, amplitude -1), U (on-site), mu (amplitude -1 per orbital of
    the cluster), optionally the Neel field M (+1 up / -1 down on sublattice A,
    opposite on B), and bath terms eb{k} (bath energies) and tb{k}
    (cluster-bath hybridization of bath k with site k % n_sites)."""
    ns = nx * ny
    no = ns + n_bath
    ops = {}
    nn, diag = _bonds_2d(nx, ny)
    ops["t"] = ("one-body", [(i, j, -1.0) for i, j in nn] + [(i + no, j + no, -1.0) for i, j in nn])
    if diag:
        ops["tp"] = ("one-body", [(i, j, -1.0) for i, j in diag]
                     + [(i + no, j + no, -1.0) for i, j in diag])
    ops["U"] = ("interaction", [(i, i + no, 1.0) for i in range(ns)])
    ops["mu"] = ("one-body", [(i, i, -1.0) for i in range(ns)] + [(i + no, i + no, -1.0) for i in range(ns)])
    if af:
        el = []
        for y in range(ny):
            for x in range(nx):
                i = x + nx * y
                s = 1.0 if (x + y) % 2 == 0 else -1.0
                el.append((i, i, s))
                el.append((i + no, i + no, -s))
        ops["M"] = ("one-body", el)
    for k in range(n_bath):
        b = ns + k
        ops[f"eb{k+1}"] = ("one-body", [(b, b, 1.0), (b + no, b + no, 1.0)])
        s = k % ns
        ops[f"tb{k+1}"] = ("one-body", [(s, b, 1.0), (s + no, b + no, 1.0)])
    return ns, n_bath, ops


ZS = [0.5j, 0.3 + 0.1j, -1.2 + 0.05j]

# Golden cases: (nx, ny, n_bath, af, params, sector, with_gf)
CASES = {
    "chain8": (8, 1, 0, False, {"t": 1.0, "U": 4.0, "mu": 2.0}, "R0:N8:S0", True),
    "chain8_n7": (8, 1, 0, False, {"t": 1.0, "U": 4.0, "mu": 2.0}, "R0:N7:S1", False),
    "ladder2x4_af": (4, 2, 0, True, {"t": 1.0, "tp": -0.3, "U": 8.0, "mu": 4.0, "M": 0.15},
                     "R0:N8:S0", True),
    "plaquette_bath4": (2, 2, 4, False,
                        {"t": 1.0, "U": 4.0, "mu": 2.0, "eb1": -1.1, "eb2": 0.7, "eb3": 1.3,
                         "eb4": -0.4, "tb1": 0.5, "tb2": 0.45, "tb3": 0.6, "tb4": 0.35},
                        "R0:N8:S0", True),
}


# Lattice golden cases.  Each: cluster sites, superlattice, lattice operators
# [(kind, name, args)], cluster-only operators from hubbard_cluster (bath),
# parameters (lattice names; cluster values 'name_1'), sector.  The chemical
# potential 'mu' is the lattice model's built-in operator (-1 per site and
# spin), as in the reference (src_qcm/lattice_model.cpp:286-295).
LATTICE_CASES = {
    "lat_chain8": dict(
        sites=[(i, 0, 0) for i in range(8)], superlattice=[(8, 0, 0)], n_bath=0,
        ops=[("inter", "U", 1.0), ("hop", "t", (1, 0, 0), -1.0, 1, 0)],
        params={"t": 1.0, "U": 4.0, "mu": 2.0}, sector="R0:N8:S0"),
    "lat_vca2x2_af": dict(
        sites=[(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0)], superlattice=[(2, 0, 0), (0, 2, 0)],
        n_bath=0,
        ops=[("inter", "U", 1.0), ("hop", "t", (1, 0, 0), -1.0, 1, 0),
             ("hop", "t", (0, 1, 0), -1.0, 1, 0), ("dw", "M", "Z", (1, 1, 0), 1.0, 0.0)],
        params={"t": 1.0, "U": 8.0, "mu": 4.0, "M": 0.0, "M_1": 0.15}, sector="R0:N4:S0"),
    "lat_cdmft2x2_b4": dict(
        sites=[(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0)], superlattice=[(2, 0, 0), (0, 2, 0)],
        n_bath=4,
        ops=[("inter", "U", 1.0), ("hop", "t", (1, 0, 0), -1.0, 1, 0),
             ("hop", "t", (0, 1, 0), -1.0, 1, 0)],
        params={"t": 1.0, "U": 4.0, "mu": 2.0, "eb1_1": -1.0, "eb2_1": 1.0, "eb3_1": -0.6,
                "eb4_1": 0.6, "tb1_1": 0.5, "tb2_1": 0.5, "tb3_1": 0.4, "tb4_1": 0.4},
        sector="R0:N8:S0"),
}
