"""The lattice layer's Fourier data of t(k) - t_c (inter-cluster elements,
H - Hc, orbital positions, wavevector map) against the reference's own
lattice model (tests/golden/lat_*.npz).  No GPU needed."""
import numpy as np
import pytest

from conftest import load_golden
from lattice_helpers import build_lattice
from models import LATTICE_CASES


@pytest.mark.parametrize("tag", list(LATTICE_CASES))
def test_fourier_data_matches_reference(tag):
    g = load_golden(tag)
    lm = build_lattice(tag)
    L = len(lm.sites)
    H, Hc = g["L_H"], g["L_Hc"]
    for spin_down in ((False, True) if H.shape[0] > L else (False,)):
        R, els, hdiff, gpos = lm.fourier(spin_down)
        sl = slice(L, 2 * L) if spin_down else slice(0, L)
        assert np.allclose(hdiff, (H - Hc)[sl, sl], atol=1e-14)
        assert np.allclose(gpos, g["L_gpos"][:L], atol=1e-14)
        if not spin_down:
            for i, K in enumerate(g["gper_k"]):  # QCM::tk takes reduced K directly
                T = hdiff.copy()
                for r, c, n, v in els:
                    T[r, c] += v * np.exp(2j * np.pi * K @ R[n])
                assert np.allclose(T, (g["tk"][i] - Hc)[:L, :L], atol=1e-14)
    d = lm.dim
    assert np.allclose(g["L_kmap"][:d, :d], lm.S[:d, :d])


def test_legendre_grid_matches_pyqcm_formula():
    from pyqcm_gb300.lattice import legendre_frequency_grid
    w, p = legendre_frequency_grid(1.0, 10.0, 4, 6, 4)
    g = load_golden("lat_vca2x2_af")
    assert np.array_equal(w, g["sef_w"]) and np.array_equal(p, g["sef_wt"])
    # the weights integrate 1/(1+w^2) over [0, inf) to pi/2 (times 1/pi)
    w, p = legendre_frequency_grid(1.0, 10.0, 40, 60, 40)
    assert abs(np.sum(p / (1 + w * w)) - 0.5) < 1e-8
