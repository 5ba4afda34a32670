"""Why the Q-matrix parity checks converged poles and G(i w_n), not every
pole: the reference against itself.  Its band Lanczos, run on one Hamiltonian
in its factorized format 'F' and in its sparse format 'S' (the same matrix,
products summed in another order; tests/golden/make_qmatrix_spread.py), gives
converged poles (|e| < 2, weight > 1e-4) that agree to ~1e-9 and G(i w_n) that
agrees to 1e-8, while the poles far from the Fermi level, which band Lanczos
never converges, differ by up to ~0.7 and even in number.  The engine is held
to the criterion the reference meets against itself
(test_oracle_golden.assert_qmatrix_parity)."""
import numpy as np
import pytest

from conftest import load_golden
from models import CASES
from test_oracle_golden import assert_qmatrix_parity

BLOCKS = [(t, q) for t in CASES if CASES[t][6] for q in ("qup", "qdn")
          if q == "qup" or CASES[t][3]]


@pytest.mark.parametrize("tag,q", BLOCKS)
def test_reference_meets_the_criterion_against_itself(tag, q):
    g = load_golden("qmatrix_spread")
    eF, vF = g[f"{tag}_F_{q}_e"], g[f"{tag}_F_{q}_v"].T
    eS, vS = g[f"{tag}_S_{q}_e"], g[f"{tag}_S_{q}_v"].T
    assert_qmatrix_parity(eF, vF, eS, vS)


def test_unconverged_poles_differ_between_the_references_two_runs():
    g = load_golden("qmatrix_spread")
    spread = 0.0
    for tag, q in BLOCKS:
        eF, vF = g[f"{tag}_F_{q}_e"], g[f"{tag}_F_{q}_v"]
        eS = g[f"{tag}_S_{q}_e"]
        w = np.sum(np.abs(vF) ** 2, axis=1)
        for e, wi in zip(eF, w):
            if not (abs(e) < 2 and wi > 1e-4):
                spread = max(spread, float(np.min(np.abs(eS - e))))
    # far above any parity tolerance: a pole-by-pole check of every pole
    # would fail for the reference against itself
    assert spread > 1e-3, spread
