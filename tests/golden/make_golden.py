"""Generates the golden fixtures in this folder by running the reference's own
exact-diagonalization code (compiled by oracle/refbuild into oracle/_ref).

Run from the repository root, in a container that has the reference tree:
    make -C oracle/refbuild && python tests/golden/make_golden.py
(`python tests/golden/make_golden.py cf` makes the continued-fraction cases only,
`... lattice` the lattice cases only, `... large [TAG ...]` the benchmarked
sectors: the 4x4 one runs the reference's serial Lanczos on 165,636,900
states, about an hour on one core.)
Each case writes <case>.npz holding the spec it ran and every array the
reference produced (see oracle/refbuild/ref_driver.cpp for the commands).
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from models import CASES, LATTICE_CASES, ZS, hubbard_cluster  # noqa: E402
sys.path.insert(0, os.path.join(ROOT))

DRIVER = os.path.join(ROOT, "oracle", "_ref", "qcm_ref_driver")
DT = {"f8": "<f8", "u4": "<u4", "u8": "<u8", "c16": "<c16"}


def run_spec(lines):
    with tempfile.TemporaryDirectory() as d:
        spec = os.path.join(d, "spec.txt")
        with open(spec, "w") as f:
            f.write("\n".join(lines) + "\n")
        subprocess.run([DRIVER, spec, d], check=True)
        out = {}
        for line in open(os.path.join(d, "manifest.txt")):
            p = line.split()
            name, dt, shape = p[0], p[1], tuple(int(s) for s in p[2:])
            a = np.fromfile(os.path.join(d, name + ".bin"), dtype=DT[dt])
            out[name] = a.reshape(shape)
        out["spec"] = np.array("\n".join(lines))
        return out


def num(x):
    """A number as the driver's stream parser reads it (numpy 2 scalars repr
    as 'np.float64(...)', which would silently parse as 0)."""
    return repr(float(x))


def model_lines(name, ns, nb, ops):
    lines = [f"model {name} {ns} {nb}"]
    for op, (typ, els) in ops.items():
        for r, c, v in els:
            lines.append(f"el {name} {op} {typ} {r} {c} {v!r}")
    return lines


def ed_case(tag, nx, ny, params, sector, n_bath=0, af=False, extra=(), gf=True, gz=()):
    ns, nb, ops = hubbard_cluster(nx, ny, n_bath, af)
    lines = ["gchar Hamiltonian_format F", "gint seed 0"]
    lines += model_lines("clus", ns, nb, ops)
    lines += [f"param {k} {v!r}" for k, v in params.items() if k in ops]
    lines += [f"instance clus {sector} 1"]
    lines += list(extra)
    if gf:
        lines += ["qmatrix 1 0 qup"]
        if af:
            lines += ["qmatrix 1 1 qdn"]
        for k, z in enumerate(gz):
            lines += [f"gz 1 0 {z.real!r} {z.imag!r} gz{k}"]
            if af:
                lines += [f"gz 1 1 {z.real!r} {z.imag!r} gzdn{k}"]
            if n_bath:
                lines += [f"hyb 1 0 {z.real!r} {z.imag!r} hyb{k}",
                          f"sigma 1 0 {z.real!r} {z.imag!r} sig{k}"]
        lines += ["omega 1 omega"]
    lines += ["gs 1 gs"]
    out = run_spec(lines)
    np.savez_compressed(os.path.join(HERE, tag + ".npz"), **out)
    print(tag, sorted(k for k in out if k != "spec"))


# Cases run again with the continued-fraction Green function (GF_method 'F'):
# G(z) on ZS from the reference's build_cf + continued_fraction_set.  The
# reference's build_cf reads H->B->dim, which its factorized format leaves
# null (src_ed/model_instance.cpp:51, a null dereference), so these run on
# its sparse format 'S': the same Hamiltonian, stored as a CSR matrix.
CF_CASES = ["chain8", "ladder2x4_af", "plaquette_bath4"]


def cf_case(tag, method="F"):
    """G(z) with GF_method F (continued fractions; sparse format, see above) or
    M (matrix continued fractions from block Lanczos; factorized format)."""
    nx, ny, nb, af, params, sec, _ = CASES[tag]
    ns, nb, ops = hubbard_cluster(nx, ny, nb, af)
    fmt = "S" if method == "F" else "F"
    lines = [f"gchar Hamiltonian_format {fmt}", f"gchar GF_method {method}", "gint seed 0"]
    lines += model_lines("clus", ns, nb, ops)
    lines += [f"param {k} {v!r}" for k, v in params.items() if k in ops]
    lines += [f"instance clus {sec} 1"]
    for k, z in enumerate(ZS):
        lines += [f"gz 1 0 {z.real!r} {z.imag!r} gz{k}"]
        if af:
            lines += [f"gz 1 1 {z.real!r} {z.imag!r} gzdn{k}"]
    lines += ["gs 1 gs"]
    out = run_spec(lines)
    suffix = "_cf" if method == "F" else "_mcf"
    np.savez_compressed(os.path.join(HERE, tag + suffix + ".npz"), **out)
    print(tag + suffix, sorted(k for k in out if k != "spec"))


# Benchmarked sectors too large for vector fixtures: the reference's serial
# factorized product on its seeded start vector, reduced to checksums and
# 4096 sampled elements (hcheck), and its Lanczos ground-state energy
# (lanczos_e0).  (nx, ny, params, sector, accur_lanczos)
LARGE_CASES = {
    # 4x4 Hubbard cluster at half filling, dim 165,636,900 (~1.3 GB per vector)
    "large_4x4": (4, 4, {"t": 1.0, "U": 8.0, "mu": 4.0}, "R0:N16:S0", 1e-10),
    # 3x4 Hubbard cluster with diagonal hopping at half filling, dim 853,776
    "large_3x4": (3, 4, {"t": 1.0, "tp": -0.3, "U": 8.0, "mu": 4.0}, "R0:N12:S0", 1e-10),
}


def large_case(tag):
    nx, ny, params, sec, acc = LARGE_CASES[tag]
    ns, nb, ops = hubbard_cluster(nx, ny)
    lines = ["gchar Hamiltonian_format F", "gint seed 0", f"gdouble accur_lanczos {acc!r}"]
    lines += model_lines("clus", ns, nb, ops)
    lines += [f"param {k} {v!r}" for k, v in params.items() if k in ops]
    lines += [f"instance clus {sec} 1", f"hcheck clus {sec} h", f"lanczos_e0 clus {sec} lz"]
    out = run_spec(lines)
    np.savez_compressed(os.path.join(HERE, tag + ".npz"), **out)
    print(tag, {k: out[k] for k in out if k != "spec" and out[k].size == 1})


def _lattice_head(ns, nb, bath_ops, sites, superlattice, ops, params, sector):
    """Spec lines of a lattice model (cluster-only bath operators, lattice
    operators, parameters, target sector, instance 0)."""
    lines = ["gchar Hamiltonian_format F", "gint seed 0", f"model clus {ns} {nb}"]
    if bath_ops:
        for op, (typ, els) in bath_ops.items():
            for r, cc, v in els:
                lines.append(f"el clus {op} {typ} {r} {cc} {v!r}")
        lines.append("ops clus")
    lines.append("lat_cluster clus " + " ".join(f"{x} {y} {z}" for x, y, z in sites))
    lines.append("lat_model L " + " ".join(" ".join(str(a) for a in v) for v in superlattice))
    for op in ops:
        if op[0] == "inter":
            lines.append(f"lat_inter {op[1]} {op[2]!r} Hubbard")
        elif op[0] == "hop":
            lx, ly, lz = op[2]
            lines.append(f"lat_hop {op[1]} {lx} {ly} {lz} {op[3]!r} {op[4]} {op[5]}")
        elif op[0] == "dw":
            qx, qy, qz = op[3]
            lines.append(f"lat_dw {op[1]} {op[2]} {qx} {qy} {qz} {op[4]!r} {op[5]!r}")
    for k, v in params.items():
        lines.append(f"lat_param {k} {v!r}")
    lines.append(f"lat_sector {sector}")
    lines.append("lat_instance 0")
    return lines


def bench_c2():
    """The VCA case on its benchmarked grid: 3x4 cluster (4 wide, 3 high),
    tiled by the superlattice (4,0), (1,3) on which the Neel wavevector is
    commensurate (the reference refuses (4,0), (0,3) for a density wave at
    (pi, pi)), t=1, t'=-0.3, U=8, mu=4, Neel Weiss field M_1=0.1; ground-state energy,
    both spin blocks' Q-matrices, the cluster part of Omega and the Potthoff
    functional on the 128x128 wavevector grid x 256 Gauss-Legendre
    frequencies (reference: QCM::Potthoff_functional, grid path)."""
    from pyqcm_gb300.lattice import legendre_frequency_grid
    sites = [(x, y, 0) for y in range(3) for x in range(4)]
    ops = [("inter", "U", 1.0), ("hop", "t", (1, 0, 0), -1.0, 1, 0),
           ("hop", "t", (0, 1, 0), -1.0, 1, 0), ("hop", "tp", (1, 1, 0), -1.0, 1, 0),
           ("hop", "tp", (-1, 1, 0), -1.0, 1, 0), ("dw", "M", "Z", (1, 1, 0), 1.0, 0.0)]
    params = {"t": 1.0, "tp": -0.3, "U": 8.0, "mu": 4.0, "M": 0.0, "M_1": 0.1}
    lines = _lattice_head(12, 0, None, sites, [(4, 0, 0), (1, 3, 0)], ops, params, "R0:N12:S0")
    w, wt = legendre_frequency_grid(1.0, 10.0, 64, 128, 64)
    lines += ["gs 0 gs", "qmatrix 0 0 qup", "qmatrix 0 1 qdn", "omega 0 omega_clus",
              "lat_kgrid 128 128 1",
              f"lat_wgrid {len(w)} " + " ".join(num(x) for x in w) + " " + " ".join(num(x) for x in wt),
              "lat_sef 0 sef"]
    out = run_spec(lines)
    out["sef_w"], out["sef_wt"] = w, wt
    np.savez_compressed(os.path.join(HERE, "bench_vca3x4.npz"), **out)
    print("bench_vca3x4", {k: out[k] for k in out if out[k].size == 1 and k != "spec"})


def plaquette_bath8_ops():
    """Bath operators of the batched-CDMFT case: 2x2 plaquette (orbitals 0..3)
    with 8 bath orbitals (4..11); bath k has energy eb{k+1} and two
    hybridizations, tb{k+1} with site k % 4 and tb{k+9} with site (k+1) % 4
    (8 energies + 16 hybridizations)."""
    ns, nb = 4, 8
    no = ns + nb
    ops = {}
    for k in range(nb):
        b = ns + k
        ops[f"eb{k+1}"] = ("one-body", [(b, b, 1.0), (b + no, b + no, 1.0)])
    for k in range(nb):
        b = ns + k
        for j, s in ((k + 1, k % ns), (k + 1 + nb, (k + 1) % ns)):
            ops[f"tb{j}"] = ("one-body", [(s, b, 1.0), (s + no, b + no, 1.0)])
    return ops


BENCH_C4_PARAMS = {"t": 1.0, "tp": 0.0, "U": 6.0, "mu": 3.0,
                   **{f"eb{k+1}_1": v for k, v in enumerate([-2.1, -1.3, -0.7, -0.2, 0.3, 0.8, 1.4, 2.2])},
                   **{f"tb{k+1}_1": v for k, v in enumerate([0.55, 0.4, 0.35, 0.5, 0.45, 0.3, 0.6, 0.25,
                                                             0.15, 0.2, 0.1, 0.12, 0.18, 0.08, 0.22, 0.05])}}


def bench_c4():
    """The batched-CDMFT model at its benchmarked grids: 2x2 plaquette + 8
    bath orbitals (plaquette_bath8_ops), sector R0:N12:S0, one parameter
    point; ground-state energy, the cluster Green function at four Matsubara
    frequencies, the CDMFT host function on the 64x64 k grid (kgrid_side)
    at the 200 Matsubara frequencies of beta = 50, and CDMFT distances at
    two bath points (reference: CDMFT_host, CDMFT_distance)."""
    sites = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0)]
    ops = [("inter", "U", 1.0), ("hop", "t", (1, 0, 0), -1.0, 1, 0),
           ("hop", "t", (0, 1, 0), -1.0, 1, 0), ("hop", "tp", (1, 1, 0), -1.0, 1, 0),
           ("hop", "tp", (-1, 1, 0), -1.0, 1, 0)]
    bops = plaquette_bath8_ops()
    lines = _lattice_head(4, 8, bops, sites, [(2, 0, 0), (0, 2, 0)], ops, BENCH_C4_PARAMS,
                          "R0:N12:S0")
    beta = 50.0
    wn = [(2 * n + 1) * np.pi / beta for n in range(200)]
    lines += ["gs 0 gs"]
    for k, n in enumerate((0, 3, 20, 199)):
        lines.append(f"gz 0 0 0.0 {num(wn[n])} gz{k}")
    lines += ["gint kgrid_side 64",
              f"lat_host 0 host {len(wn)} " + " ".join(num(x) for x in wn) + " "
              + " ".join("1.0" for _ in wn)]
    names = [f"eb{k+1}_1" for k in range(8)] + [f"tb{k+1}_1" for k in range(16)]
    lines.append("lat_varia " + " ".join(names))
    p0 = [BENCH_C4_PARAMS[n] for n in names]
    p1 = [v * 1.05 + 0.01 for v in p0]
    lines.append(f"lat_dist 0 dist0 {len(p0)} " + " ".join(num(x) for x in p0))
    lines.append(f"lat_dist 0 dist1 {len(p1)} " + " ".join(num(x) for x in p1))
    out = run_spec(lines)
    out["host_w"] = np.array(wn)
    out["gz_n"] = np.array([0, 3, 20, 199])
    out["dist_p0"], out["dist_p1"] = np.array(p0), np.array(p1)
    np.savez_compressed(os.path.join(HERE, "bench_cdmft2x2_b8.npz"), **out)
    print("bench_cdmft2x2_b8", {k: out[k] for k in out if out[k].size == 1 and k != "spec"})


def main():
    if sys.argv[1:2] == ["bench"]:  # the benchmarked lattice cases (C2 VCA, C4 CDMFT)
        which = sys.argv[2:] or ["c2", "c4"]
        if "c2" in which:
            bench_c2()
        if "c4" in which:
            bench_c4()
        return
    if not os.path.exists(DRIVER):
        sys.exit("build the reference oracle first: make -C oracle/refbuild")
    if sys.argv[1:2] == ["large"]:  # large_<case> [...]: the benchmarked sectors
        for tag in sys.argv[2:] or list(LARGE_CASES):
            large_case(tag)
        return
    if sys.argv[1:] == ["lattice"]:  # the lattice cases only
        for tag, c in LATTICE_CASES.items():
            lattice_case(tag, c)
        return
    if sys.argv[1:] == ["cf"]:  # the (matrix) continued-fraction cases only
        for tag in CF_CASES:
            cf_case(tag)
            cf_case(tag, "M")
        return
    # Half bases for L = 8, 12, 16 at half filling and one off-half filling.
    lines = ["halfbasis 8 4", "halfbasis 8 3", "halfbasis 12 6", "halfbasis 12 5", "halfbasis 16 8"]
    out = run_spec(lines)
    np.savez_compressed(os.path.join(HERE, "halfbasis.npz"), **out)
    for tag, (nx, ny, nb, af, params, sec, gf) in CASES.items():
        extra = [f"hamiltonian clus {sec} h", f"lanczos clus {sec} lz"]
        if tag == "chain8":
            extra += [f"destroy clus {sec} 3 0 -1 dup", f"destroy clus {sec} 5 1 -1 ddn",
                      f"destroy clus {sec} 2 0 1 cup", f"destroy clus {sec} 6 1 1 cdn"]
        ed_case(tag, nx, ny, params, sec, n_bath=nb, af=af, extra=extra, gf=gf, gz=ZS)
    for tag, c in LATTICE_CASES.items():
        lattice_case(tag, c)
    for tag in CF_CASES:
        cf_case(tag)
        cf_case(tag, "M")

def lattice_case(tag, c):
    """Runs a lattice model through the reference's QCM layer."""
    from pyqcm_gb300.lattice import legendre_frequency_grid
    ns = len(c["sites"])
    nb = c["n_bath"]
    lines = ["gchar Hamiltonian_format F", "gint seed 0", f"model clus {ns} {nb}"]
    if nb:
        _, _, bops = hubbard_cluster(2, 2, nb)
        for op, (typ, els) in bops.items():
            if op.startswith("eb") or op.startswith("tb"):
                for r, cc, v in els:
                    lines.append(f"el clus {op} {typ} {r} {cc} {v!r}")
        lines.append("ops clus")
    lines.append("lat_cluster clus " + " ".join(f"{x} {y} {z}" for x, y, z in c["sites"]))
    lines.append("lat_model L " + " ".join(" ".join(str(a) for a in v) for v in c["superlattice"]))
    for op in c["ops"]:
        if op[0] == "inter":
            lines.append(f"lat_inter {op[1]} {op[2]!r} Hubbard")
        elif op[0] == "hop":
            lx, ly, lz = op[2]
            lines.append(f"lat_hop {op[1]} {lx} {ly} {lz} {op[3]!r} {op[4]} {op[5]}")
        elif op[0] == "dw":
            qx, qy, qz = op[3]
            lines.append(f"lat_dw {op[1]} {op[2]} {qx} {qy} {qz} {op[4]!r} {op[5]!r}")
    for k, v in c["params"].items():
        lines.append(f"lat_param {k} {v!r}")
    lines.append(f"lat_sector {c['sector']}")
    lines.append("lat_instance 0")
    dim = len(c["superlattice"])
    ks = [(0.0, 0.0, 0.0), (0.125, 0.0, 0.0), (0.25, 0.0, 0.0), (0.5, 0.0, 0.0)]
    if dim == 2:
        ks = [(0.0, 0.0, 0.0), (0.125, 0.25, 0.0), (0.25, 0.25, 0.0), (0.5, 0.0, 0.0)]
    zs = [0.5 + 0.1j, -1.0 + 0.1j, 2.0 + 0.1j, 0.3j]
    lines.append(f"lat_gper 0 gper {len(zs)} " + " ".join(f"{z.real!r} {z.imag!r}" for z in zs)
                 + f" {len(ks)} " + " ".join(f"{a!r} {b!r} {d!r}" for a, b, d in ks))
    lines.append("lat_dump 0 L")
    lines.append(f"lat_tk 0 tk {len(ks)} " + " ".join(f"{a!r} {b!r} {d!r}" for a, b, d in ks))
    w, wt = legendre_frequency_grid(1.0, 10.0, 4, 6, 4)
    lines.append(f"lat_kgrid 8 {8 if dim >= 2 else 1} 1")
    lines.append(f"lat_wgrid {len(w)} " + " ".join(num(x) for x in w) + " "
                 + " ".join(num(x) for x in wt))
    lines.append("lat_sef 0 sef")
    dos_z = [complex(x, 0.1) for x in (-3.0, -1.0, -0.2, 0.0, 0.5, 2.0)]
    lines.append(f"lat_dos 0 dos {len(dos_z)} " + " ".join(f"{z.real!r} {z.imag!r}" for z in dos_z))
    ave_ops = [op[1] for op in c["ops"] if op[0] in ("hop", "dw")]
    ave_ops = list(dict.fromkeys(ave_ops)) + ["mu"]
    lines.append("lat_ave 0 ave " + " ".join(ave_ops))
    lines.append("lat_pe 0 epot")
    lines.append("omega 0 omega_clus")
    if nb:
        beta = 50.0
        wn = [(2 * n + 1) * np.pi / beta for n in range(20)]
        lines.append("gint kgrid_side 8")
        lines.append(f"lat_host 0 host {len(wn)} " + " ".join(num(x) for x in wn) + " "
                     + " ".join("1.0" for _ in wn))
        lines.append("lat_varia eb1_1 eb2_1 tb1_1")
        lines.append("lat_dist 0 dist0 3 -1.0 1.0 0.5")
        lines.append("lat_dist 0 dist1 3 -1.2 0.8 0.45")
    out = run_spec(lines)
    out["sef_w"] = w
    out["sef_wt"] = wt
    out["gper_k"] = np.array(ks)
    out["gper_z"] = np.array(zs)
    out["dos_z"] = np.array(dos_z)
    out["ave_ops"] = np.array(ave_ops)
    np.savez_compressed(os.path.join(HERE, tag + ".npz"), **out)
    print(tag, sorted(k for k in out if k != "spec"))


if __name__ == "__main__":
    main()
