"""Host eigensolvers of band Lanczos (pyqcm_gb300/csrc/qcmg_tridiag.cpp),
compiled on their own with the host C++ compiler and checked against
numpy's dense symmetric eigensolver:
- band_lowest: the convergence probe (lowest eigenvalue of the projected
  band matrix, Lanczos.hpp:338-362);
- band_eigen_leading: all eigenvalues and the leading p rows of the
  eigenvectors, from which the Q-matrix is formed
  (Hamiltonian_base.hpp:229-254).  Eigenvector signs and bases of
  degenerate eigenspaces are arbitrary, so the rows are compared through
  the resolvent of the leading block, W (z - E)^-1 W^T, which is what the
  Green function uses."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "pyqcm_gb300", "csrc")

DRIVER = r"""
#include "qcmg_tridiag.h"
#include <cstdio>
#include <vector>
int main() {
  int n, ld, b, p;
  while (std::scanf("%d %d %d %d", &n, &ld, &b, &p) == 4) {
    std::vector<double> t((size_t)ld * n);
    for (double& v : t) std::scanf("%lf", &v);
    std::vector<double> ev, W;
    const double lo = qcmg::band_lowest(t, ld, n, b);
    // hinted: from just above, and from a wrong hint far above and below
    const double lo_near = qcmg::band_lowest(t, ld, n, b, lo + 1e-9, 1e-6);
    const double lo_high = qcmg::band_lowest(t, ld, n, b, lo + 3.0, 1e-9);
    const double lo_low = qcmg::band_lowest(t, ld, n, b, lo - 3.0, 1e-9);
    const bool ok = qcmg::band_eigen_leading(t, ld, n, b, p, ev, W);
    std::printf("%d %.17g %.17g %.17g %.17g\n", ok ? 1 : 0, lo, lo_near, lo_high, lo_low);
    for (double v : ev) std::printf("%.17g\n", v);
    for (double v : W) std::printf("%.17g\n", v);
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("band_eigen")
    src = d / "driver.cpp"
    src.write_text(DRIVER)
    exe = d / "driver"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, str(src),
                    os.path.join(CSRC, "qcmg_tridiag.cpp"), "-o", str(exe)], check=True)
    return str(exe)


def _band(rng, n, b, diag=None):
    A = np.zeros((n, n))
    for k in range(b + 1):
        v = rng.normal(size=n - k) * (2.0 if k == 0 else 1.0)
        A += np.diag(v, -k) + (np.diag(v, k) if k else 0)
    if diag is not None:
        A[np.diag_indices(n)] = diag
    return A


def _run(driver, mats):
    """mats: list of (A, b, p); t is passed column-major with ld = n + 3 and
    only its lower band filled, as band Lanczos holds it."""
    lines = []
    for A, b, p in mats:
        n = A.shape[0]
        ld = n + 3
        t = np.zeros((n, ld))  # t[c, r] = A[r, c] for r >= c within the band
        for c in range(n):
            for r in range(c, min(n, c + b + 1)):
                t[c, r] = A[r, c]
        lines.append(f"{n} {ld} {b} {p}")
        lines.extend(f"{v:.17g}" for v in t.ravel())
    out = subprocess.run([driver], input="\n".join(lines) + "\n", capture_output=True, text=True,
                         check=True).stdout.split()
    res, o = [], 0
    for A, b, p in mats:
        n = A.shape[0]
        ok, lo = int(out[o]), np.array(out[o + 1:o + 5], float)
        o += 5
        ev = np.array(out[o:o + n], float)
        o += n
        W = np.array(out[o:o + p * n], float).reshape(p, n)
        o += p * n
        res.append((ok, lo, ev, W))
    return res


CASES = [(1, 0, 1), (2, 1, 2), (5, 2, 3), (40, 3, 4), (97, 4, 4), (200, 4, 8), (150, 12, 12),
         (60, 1, 3)]


def test_band_solvers_against_numpy(driver):
    rng = np.random.default_rng(11)
    mats = []
    for n, b, p in CASES:
        mats.append((_band(rng, n, b), b, p))
    # a repeated diagonal gives near-degenerate clusters
    mats.append((_band(rng, 60, 2, diag=(np.arange(60) % 3) - 1.0), 2, 4))
    # an exactly degenerate lowest eigenvalue (two uncoupled copies of one block)
    B = _band(rng, 30, 3)
    D = np.zeros((60, 60))
    D[::2, ::2] = B
    D[1::2, 1::2] = B
    mats.append((D, 7, 4))
    for (A, b, p), (ok, lo, ev, W) in zip(mats, _run(driver, mats)):
        n = A.shape[0]
        w, V = np.linalg.eigh(A)
        scale = np.abs(A).max()
        assert ok
        assert np.max(np.abs(lo - w[0])) <= 1e-13 * scale, (n, b, lo - w[0])
        assert np.max(np.abs(ev - w)) <= 1e-13 * scale, (n, b)
        k = min(p, n)
        assert np.max(np.abs(W[:k] @ W[:k].T - np.eye(k))) < 1e-13
        for z in (0.3 + 0.7j, -1.1 + 0.2j, 2.0 + 1.5j):
            R = (W[:k] / (z - ev)) @ W[:k].T
            Rref = (V[:k] / (z - w)) @ V[:k].T
            assert np.max(np.abs(R - Rref)) < 1e-12, (n, b, z)


def test_diagonal_band_matrix(driver):
    """b = 0: the eigenvectors are unit vectors, sorted with the diagonal."""
    d = np.array([3.0, -1.0, 2.0, -5.0, 0.5])
    [(ok, lo, ev, W)] = _run(driver, [(np.diag(d), 0, 2)])
    assert ok and lo == pytest.approx(-5.0, abs=1e-15)
    assert np.array_equal(ev, np.sort(d))
    order = np.argsort(d)
    assert np.array_equal(np.abs(W), np.abs(np.eye(5)[:2, order]))
