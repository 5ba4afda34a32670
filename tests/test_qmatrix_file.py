"""Q-matrix files (ModelInstance.write_qmatrix / read_qmatrix): the round
trip of the Lehmann data on the host, and the refusal of a file written for
other parameter values."""
import numpy as np
import pytest


def _instance(U=4.0):
    import pyqcm_gb300 as pg
    m = pg.ClusterModel(n_sites=2)
    m.new_operator("t", "one-body", [(0, 1, -1.0), (2, 3, -1.0)])
    m.new_operator("U", "interaction", [(0, 2, 1.0), (1, 3, 1.0)])
    return pg.ModelInstance(m, {"t": 1.0, "U": U}, "R0:N2:S0")


def _fake_solution(inst, rng):
    from pyqcm_gb300.ed import Sector, State
    states = []
    for sec, en, w in (("R0:N2:S0", -2.1, 0.75), ("R0:N2:S2", -2.0, 0.25)):
        st = State(Sector(sec), en, None)
        st.weight = w
        st.gf = (rng.normal(size=5), rng.normal(size=(2, 5)) + 1j * rng.normal(size=(2, 5)))
        st.gf_down = (rng.normal(size=3), rng.normal(size=(2, 3)) + 0j)
        states.append(st)
    inst.states, inst.mixing = states, 4
    inst.GS_energy, inst.E0 = -2.1, -2.075
    inst.gs_solved = inst.gf_solved = True


def test_qmatrix_file_round_trip(tmp_path):
    a = _instance()
    _fake_solution(a, np.random.default_rng(3))
    path = tmp_path / "q.npz"
    a.write_qmatrix(path)
    b = _instance()
    b.read_qmatrix(path)
    assert b.gs_solved and b.gf_solved and b.mixing == 4
    assert (b.GS_energy, b.E0) == (a.GS_energy, a.E0)
    assert len(b.states) == len(a.states)
    for sa, sb in zip(a.states, b.states):
        assert sb.sec.name() == sa.sec.name() and (sb.energy, sb.weight) == (sa.energy, sa.weight)
        for blk in ("gf", "gf_down"):
            (ea, va), (eb, vb) = getattr(sa, blk), getattr(sb, blk)
            assert np.array_equal(ea, eb) and np.array_equal(va, vb)


def test_qmatrix_file_for_other_parameters_is_refused(tmp_path):
    a = _instance(U=4.0)
    _fake_solution(a, np.random.default_rng(4))
    path = tmp_path / "q.npz"
    a.write_qmatrix(path)
    with pytest.raises(ValueError):
        _instance(U=5.0).read_qmatrix(path)
