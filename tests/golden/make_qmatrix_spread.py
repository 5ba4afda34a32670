"""Evidence for the Q-matrix parity criterion: the reference's own band
Lanczos run twice on the same Hamiltonian, once in its factorized format 'F'
and once in its sparse format 'S' (the same matrix, products summed in another
order), for the golden cases with a Green function.  Writes
qmatrix_spread.npz: both runs' poles and weights per case and spin block.

Run from the repository root where the reference oracle is built:
    make -C oracle/refbuild && python tests/golden/make_qmatrix_spread.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import model_lines, run_spec  # noqa: E402
from models import CASES, hubbard_cluster  # noqa: E402


def run(tag, fmt):
    nx, ny, nb, af, params, sec, _ = CASES[tag]
    ns, nb, ops = hubbard_cluster(nx, ny, nb, af)
    lines = [f"gchar Hamiltonian_format {fmt}", "gint seed 0"]
    lines += model_lines("clus", ns, nb, ops)
    lines += [f"param {k} {v!r}" for k, v in params.items() if k in ops]
    lines += [f"instance clus {sec} 1", "qmatrix 1 0 qup"]
    if af:
        lines += ["qmatrix 1 1 qdn"]
    return run_spec(lines)


def main():
    out = {}
    for tag in [t for t in CASES if CASES[t][6]]:
        for fmt in ("F", "S"):
            r = run(tag, fmt)
            for k, v in r.items():
                if k != "spec":
                    out[f"{tag}_{fmt}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "qmatrix_spread.npz"), **out)
    print(sorted(out))


if __name__ == "__main__":
    main()
