"""Checkpoint files (ib_checkpoint_save / ib_checkpoint_load) through the C ABI.

* An FP64 run restarted from a checkpoint on a new handle continues to the same bits as the
  uninterrupted run (static bodies; moving bodies with the CG warm start's history restored).
* The oracle continues a run from a checkpoint the GPU wrote, within the FP64 parity bars.
* A checkpoint of another grid is refused.
"""
import numpy as np
import pytest

from _util import oracle_problem, rel

pytestmark = pytest.mark.gpu


def _start(ib, wl, precision="fp64", moving=False):
    prob = wl.problem()
    st = ib.initstate(prob)
    st._gamma[:] = wl.initial_gamma()
    s = ib.initsolver(prob, st, precision=precision)
    if moving:
        s.set_cg_options(tol=1e-12, warm_start="extrapolate")
    s.vort2flux(st)
    return prob, st, s


def test_restart_continues_to_the_same_bits(ib, tmp_path):
    wl = ib.workloads.scaled(ib.workloads.two_body_large(), 128, 128, nlevels=3)
    prob, st, s = _start(ib, wl)
    for i in range(6):
        ib.advance_(st, s, i * wl.dt)
    path = tmp_path / "run.ckpt"
    s.save_checkpoint(path)
    for i in range(6, 10):
        ib.advance_(st, s, i * wl.dt)
    want_g, want_f = st.qty.gamma.copy(), st.qty.Fb.copy()
    want_cd, _ = s.force_history(4)
    # a fresh handle of the same problem, from the file
    prob2, st2, s2 = _start(ib, wl)
    s2.load_checkpoint(path, st2)
    assert st2.t == pytest.approx(5 * wl.dt)
    for i in range(6, 10):
        ib.advance_(st2, s2, i * wl.dt)
    np.testing.assert_array_equal(st2.qty.gamma, want_g)
    np.testing.assert_array_equal(st2.qty.Fb, want_f)
    cd2, _ = s2.force_history(4)
    np.testing.assert_array_equal(cd2, want_cd)
    s.close()
    s2.close()


def test_moving_restart_continues_to_the_same_bits(ib, tmp_path):
    base = ib.workloads.heaving_plate(nsteps=10)
    wl = ib.workloads.scaled(base, 128, 96, nlevels=2, nsteps=10)
    wl.Re, wl.dt = 200.0, 0.01
    prob, st, s = _start(ib, wl, moving=True)
    for i in range(5):
        ib.advance_(st, s, i * wl.dt)
    path = tmp_path / "moving.ckpt"
    s.save_checkpoint(path)
    for i in range(5, 8):
        ib.advance_(st, s, i * wl.dt)
    want_g, want_f = st.qty.gamma.copy(), st.qty.Fb.copy()
    prob2, st2, s2 = _start(ib, wl, moving=True)
    s2.load_checkpoint(path, st2)
    for i in range(5, 8):
        ib.advance_(st2, s2, i * wl.dt)
    np.testing.assert_array_equal(st2.qty.gamma, want_g)
    np.testing.assert_array_equal(st2.qty.Fb, want_f)
    s.close()
    s2.close()


def test_oracle_continues_from_a_gpu_checkpoint(ib, O, tmp_path):
    wl = ib.workloads.scaled(ib.workloads.cylinder_small(), 64, 64, nlevels=2)
    prob, st, s = _start(ib, wl)
    for i in range(5):
        ib.advance_(st, s, i * wl.dt)
    path = tmp_path / "c.ckpt"
    s.save_checkpoint(path)
    op = oracle_problem(O, wl, prob)
    ck = O.read_checkpoint(path, op.grid)
    assert ck["steps"] == 5 and ck["t"] == pytest.approx(4 * wl.dt)
    ost = O.state_from_checkpoint(op, ck)
    osol = O.Solver(op)
    for i in range(5, 8):
        ib.advance_(st, s, i * wl.dt)
        osol.advance(ost, i * wl.dt)
        assert rel(st.qty.gamma, ost.gamma.reshape(op.grid.nlevels, -1)) < 1e-10
        assert abs(st.qty.stress[0].CD - ost.cd[0]) / max(1.0, abs(ost.cd[0])) < 1e-8
    s.close()


def test_checkpoint_of_another_grid_is_refused(ib, tmp_path):
    wl = ib.workloads.scaled(ib.workloads.cylinder_small(), 64, 64, nlevels=2)
    _, st, s = _start(ib, wl)
    path = tmp_path / "c.ckpt"
    s.save_checkpoint(path)
    wl2 = ib.workloads.scaled(ib.workloads.cylinder_small(), 96, 96, nlevels=2)
    _, st2, s2 = _start(ib, wl2)
    with pytest.raises(Exception, match="checkpoint"):
        s2.load_checkpoint(path, st2)
    s.close()
    s2.close()


def test_mixed_restart_stays_within_the_mixed_bars(ib, tmp_path):
    """A mixed-precision handle restarts from its checkpoint (float-float state stored as FP64,
    the refinement predictors restart from zero) within the mixed bars of the uninterrupted run:
    Gamma 1e-8 (relative L2), C_D / C_L 1e-6."""
    wl = ib.workloads.scaled(ib.workloads.two_body_large(), 128, 128, nlevels=3)
    prob, st, s = _start(ib, wl, precision="mixed")
    for i in range(6):
        ib.advance_(st, s, i * wl.dt)
    path = tmp_path / "mixed.ckpt"
    s.save_checkpoint(path)
    for i in range(6, 12):
        ib.advance_(st, s, i * wl.dt)
    want_g = st.qty.gamma.copy()
    want_c = [(b.CD, b.CL) for b in st.qty.stress]
    prob2, st2, s2 = _start(ib, wl, precision="mixed")
    s2.load_checkpoint(path, st2)
    for i in range(6, 12):
        ib.advance_(st2, s2, i * wl.dt)
    assert rel(st2.qty.gamma, want_g) < 1e-8
    for (cd, cl), b in zip(want_c, st2.qty.stress):
        assert abs(b.CD - cd) / max(1.0, abs(cd)) < 1e-6 and abs(b.CL - cl) / max(1.0, abs(cl)) < 1e-6
    s.close()
    s2.close()
