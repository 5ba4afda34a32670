"""Generates the golden fixtures in this folder by running the reference's own
exact-diagonalization code (compiled by oracle/refbuild into oracle/_ref).

Run from the repository root, in a container that has the reference tree:
    make -C oracle/refbuild && python tests/golden/make_golden.py
(`python tests/golden/make_golden.py cf` makes the continued-fraction cases only,
`... lattice` the lattice cases only.)
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
DT = {"f8": "<f8", "u4": "<u4", "c16": "<c16"}


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


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference oracle first: make -C oracle/refbuild")
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
