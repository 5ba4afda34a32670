"""Calibrates the CPU port against the reference's own code: the
reference's serial Hamiltonian_Factorized::mult_add (pyqcm
src_ed/Hamiltonian/Hamiltonian_Factorized.hpp, built from its sources into
oracle/_ref) and the port's product (qcm_oracle.Sector.mult_add, one
thread) on the same 4x4 N=16 Sz=0 sector (165,636,900 states), on the
same host, one after the other.  Writes oracle/port_calibration.json:
seconds per product of each (median of `--repeats`), their ratio, and the
host.  The reference's product has no threading, so its serial time is its
time on any core count.

Needs the reference oracle (make -C oracle/refbuild); run from the
repository root:  python oracle/calibrate_port.py
"""
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
sys.path.insert(0, ROOT)


def reference_seconds(repeats):
    from make_golden import LARGE_CASES, hubbard_cluster, model_lines, run_spec
    nx, ny, params, sec, acc = LARGE_CASES["large_4x4"]
    ns, nb, ops = hubbard_cluster(nx, ny)
    lines = ["gchar Hamiltonian_format F", "gint seed 0"]
    lines += model_lines("clus", ns, nb, ops)
    lines += [f"param {k} {v!r}" for k, v in params.items() if k in ops]
    lines += [f"instance clus {sec} 1"] + [f"hcheck clus {sec} h{r}" for r in range(repeats)]
    out = run_spec(lines)
    return [float(out[f"h{r}_mult_add_s"]) for r in range(repeats)], int(out["h0_dim"])


def port_seconds(repeats):
    import bench
    import qcm_oracle as qo
    ns, nb, ops = bench.model_ops()
    up, dn, pr = qo.combine_terms(ops, bench.PARAMS, ns)
    _, nup, ndn = bench.sector_of(4, 4)
    S = qo.Sector(ns, nup, ndn, up, dn, pr)
    x = qo.seeded_start(S.dim)
    y = np.zeros(S.dim)
    S.mult_add(x, y, nthreads=1)  # page faults
    ts = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        S.mult_add(x, y, nthreads=1)
        ts.append(time.perf_counter() - t0)
    return ts, S.dim


def main():
    repeats = int(sys.argv[sys.argv.index("--repeats") + 1]) if "--repeats" in sys.argv else 3
    tr, dim_r = reference_seconds(repeats)
    tp, dim_p = port_seconds(repeats)
    assert dim_r == dim_p, (dim_r, dim_p)
    out = {"sector": "4x4 Hubbard cluster t=1 U=8 mu=4, R0:N16:S0", "dim": dim_p,
           "reference_mult_add_s": float(np.median(tr)), "reference_runs_s": tr,
           "port_mult_add_1thread_s": float(np.median(tp)), "port_runs_s": tp,
           "port_over_reference_speed": float(np.median(tr) / np.median(tp)),
           "host": f"{platform.machine()}, {os.cpu_count()} cores, {platform.processor() or ''}"}
    with open(os.path.join(HERE, "port_calibration.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
