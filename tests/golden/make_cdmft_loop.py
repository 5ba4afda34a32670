"""The reference's CDMFT loop, run on the CPU with the reference's own C++
(oracle/_ref driven interactively): for the 4-bath plaquette golden case,
each step sets the bath, makes a new lattice model instance, builds the host
function (QCM::CDMFT_host) and fits the bath with SciPy's least_squares
('trf') on the reference's residuals and finite-difference Jacobian
(QCM::CDMFT_residuals / CDMFT_gradient), as pyqcm.cdmft.CDMFT.CDMFT_step does
with method='trf' (pyqcm/cdmft.py:479-628, optimize at :1539); the outer
iteration is the fixed point with the depth-2 'parameters' test.  Writes
cdmft_loop_b4.npz (the iterates, the converged bath, the tolerances).

Run from the repository root where the reference oracle is built:
    make -C oracle/refbuild && python tests/golden/make_cdmft_loop.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np
import scipy.optimize

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)
from make_golden import DRIVER, _lattice_head, num  # noqa: E402
from models import LATTICE_CASES, hubbard_cluster  # noqa: E402

VARIA = ["eb1_1", "eb2_1", "eb3_1", "eb4_1", "tb1_1", "tb2_1", "tb3_1", "tb4_1"]
TOL = {"accur": 1e-8, "accur_bath": 1e-12, "accur_dist": 1e-15, "depth": 2, "maxiter": 100}


class Driver:
    def __init__(self, d):
        self.p = subprocess.Popen([DRIVER, "-", d], stdin=subprocess.PIPE,
                                  stdout=subprocess.PIPE, text=True)

    def __call__(self, line):
        self.p.stdin.write(line + "\n")
        self.p.stdin.flush()
        out = None
        while True:
            s = self.p.stdout.readline()
            if not s:
                raise RuntimeError("reference driver stopped at: " + line[:80])
            s = s.strip()
            if s == "@@":
                return out
            if s.startswith("R "):
                out = np.array([float(v) for v in s.split()[2:]])

    def close(self):
        self.p.stdin.close()
        self.p.wait()


def main():
    c = LATTICE_CASES["lat_cdmft2x2_b4"]
    _, _, bops = hubbard_cluster(2, 2, 4)
    bath = {k: v for k, v in bops.items() if k.startswith("eb") or k.startswith("tb")}
    head = _lattice_head(4, 4, bath, c["sites"], c["superlattice"], c["ops"], c["params"],
                         c["sector"])
    beta = 50.0
    wn = [(2 * n + 1) * np.pi / beta for n in range(20)]
    wline = f"{len(wn)} " + " ".join(num(x) for x in wn) + " " + " ".join("1.0" for _ in wn)
    with tempfile.TemporaryDirectory() as d:
        drv = Driver(d)
        for line in head + ["gint kgrid_side 8", "lat_varia " + " ".join(VARIA)]:
            drv(line)
        x = np.array([c["params"][v] for v in VARIA])
        hist, prev = [x.copy()], []
        label = 0
        for it in range(TOL["maxiter"]):
            for v, xv in zip(VARIA, x):
                drv(f"lat_set {v} {num(xv)}")
            label += 1
            drv(f"lat_instance {label}")
            drv(f"lat_host {label} host{label} {wline}")
            F = lambda p, L=label: drv(f"lat_resid {L} {len(p)} " + " ".join(num(v) for v in p))

            def J(p, L=label):
                g = drv(f"lat_grad {L} {len(p)} " + " ".join(num(v) for v in p))
                return g.reshape(-1, len(p))
            xs = scipy.optimize.least_squares(F, x, jac=J, method="trf",
                                              ftol=TOL["accur_dist"], xtol=TOL["accur_bath"],
                                              gtol=1e-12, max_nfev=2000).x
            hist.append(xs.copy())
            # the 'parameters' test of depth 2 (pyqcm/cdmft.py:14-106)
            conv = len(prev) >= TOL["depth"] and all(
                np.linalg.norm(xs - y) / len(xs) <= TOL["accur"] for y in prev)
            prev = (prev + [xs])[-TOL["depth"]:]
            x = xs
            print(f"step {it + 1}: {x}")
            if conv:
                break
        drv.close()
    np.savez_compressed(os.path.join(HERE, "cdmft_loop_b4.npz"), x=x, history=np.array(hist),
                        iterations=it + 1, varia=np.array(VARIA),
                        **{k: v for k, v in TOL.items()})
    print("converged bath", x, "after", it + 1, "steps")


if __name__ == "__main__":
    main()
