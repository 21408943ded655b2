"""Moving bodies (RigidBody{RelativeFrame}): device kinematics, weights rebuilt every step and the
Schur solve by device CG, against the corrected moving-body oracle.

Both sides run CG to ||r|| <= 1e-13 ||rhs|| so the comparison measures arithmetic rather than
where each CG stopped (at 1e-10 the two stopping points may differ by ~tol * cond(B))."""
import numpy as np
import pytest

from _util import oracle_moving_problem, rel

pytestmark = pytest.mark.gpu

TOL_CG = 1e-13


def small_heaving(ib, nx=128, ny=96, L=2, nsteps=8):
    base = ib.workloads.heaving_plate(nsteps=nsteps)
    wl = ib.workloads.scaled(base, nx, ny, nlevels=L, nsteps=nsteps)
    wl.Re = 200.0
    wl.dt = 0.01
    return wl


@pytest.mark.parametrize("precision,gtol,ctol", [("fp64", 1e-10, 1e-8), ("mixed", 1e-8, 1e-6)])
def test_moving_plate_parity(ib, O, precision, gtol, ctol):
    wl = small_heaving(ib)
    prob = wl.problem()
    st = ib.initstate(prob)
    st._gamma[:] = wl.initial_gamma()
    s = ib.initsolver(prob, st, precision=precision)
    s.set_cg_options(tol=TOL_CG, maxiter=5000)
    s.vort2flux(st)
    op = oracle_moving_problem(O, wl, prob, TOL_CG)
    g = op.grid
    ost = O.init_state(op)
    ost.gamma[0] = wl.initial_gamma()[0].reshape(g.gshape)
    ost.psi, ost.q = O.vort2flux(ost.gamma, g, O.lap_eigs(g))
    osol = O.MovingSolver(op)
    worst_c = 0.0
    for i in range(wl.nsteps):
        t = i * wl.dt
        ib.advance_(st, s, t)
        osol.advance(ost, t)
        cd = st.qty.stress[0].CD
        cl = st.qty.stress[0].CL
        worst_c = max(worst_c, abs(cd - ost.cd[0]) / max(1, abs(ost.cd[0])),
                      abs(cl - ost.cl[0]) / max(1, abs(ost.cl[0])))
    xb, vb = st.qty.points
    np.testing.assert_allclose(xb, ost.points, rtol=0, atol=1e-14)
    np.testing.assert_allclose(vb, ost.velocities, rtol=0, atol=1e-14)
    assert rel(st.qty.gamma, ost.gamma.reshape(g.nlevels, -1)) < gtol
    assert worst_c < ctol, worst_c
    it, res = s.cg_stats(wl.nsteps)
    assert np.all(res <= TOL_CG) and np.all(it > 0)
    s.close()


def test_warm_starts_converge_and_save_iterations(ib):
    """Every warm start reaches the same residual; starting from the previous Fb (the
    reference's cg! on qty.Fb) takes fewer iterations than starting from zero."""
    wl = small_heaving(ib, nsteps=12)
    counts = {}
    for mode in ("zero", "previous", "extrapolate"):
        prob = wl.problem()
        st = ib.initstate(prob)
        s = ib.initsolver(prob, st)
        s.set_cg_options(tol=1e-10, warm_start=mode)
        ib.solve_(st, prob, (0.0, (wl.nsteps - 1) * wl.dt), solver=s)
        it, res = s.cg_stats(wl.nsteps)
        assert np.all(res <= 1e-10)
        counts[mode] = int(it[4:].sum())
        s.close()
    assert counts["previous"] < counts["zero"], counts


def test_cg_cap_is_reported(ib):
    wl = small_heaving(ib, nsteps=1)
    prob = wl.problem()
    st = ib.initstate(prob)
    s = ib.initsolver(prob, st)
    s.set_cg_options(tol=1e-14, maxiter=3)
    with pytest.raises(ib.IBError) as e:
        ib.advance_(st, s, 0.0)
    assert e.value.status == 6
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_schur_preconditioned_cg_same_answer_fewer_iterations(ib, precision):
    """PCG with the inverse Schur matrix of the first step's configuration reaches the same
    solution (both runs to ||r|| <= 1e-12 ||rhs||) in far fewer iterations than plain CG."""
    wl = small_heaving(ib, nsteps=12)
    wl.dt = 0.005  # a stable step for this motion beyond a few steps
    out = {}
    for pc in ("none", "schur_ref"):
        prob = wl.problem()
        st = ib.initstate(prob)
        st._gamma[:] = wl.initial_gamma()
        s = ib.initsolver(prob, st, precision=precision)
        s.set_cg_options(tol=1e-12, warm_start="extrapolate")
        s.set_cg_preconditioner(pc)
        s.vort2flux(st)
        for i in range(wl.nsteps):
            ib.advance_(st, s, i * wl.dt)
        it, res = s.cg_stats(wl.nsteps)
        assert np.all(res <= 1e-12)
        out[pc] = (st.qty.gamma.copy(), st.qty.Fb.copy(), int(it.sum()), s.cg_preconditioner_stats())
        s.close()
    assert rel(out["schur_ref"][0], out["none"][0]) < 1e-9
    assert rel(out["schur_ref"][1], out["none"][1]) < 1e-7
    assert out["schur_ref"][3][0] >= 1
    assert out["schur_ref"][2] < 0.5 * out["none"][2], (out["schur_ref"][2], out["none"][2])


@pytest.mark.parametrize("precision,grid", [("fp64", (128, 96, 2)), ("mixed", (128, 96, 2)),
                                            ("mixed", (128, 128, 3))])
def test_captured_moving_step_equals_eager(ib, monkeypatch, precision, grid):
    """From the third step on a moving step runs as a captured graph with the CG loop driven
    on the device; it gives the eager step's iterates (IBGB300_NO_GRAPH=1) exactly.  The
    128 x 128 grid takes the one-warp line passes and the all-levels Vort2Flux inside the loop."""
    nx, ny, L = grid
    wl = small_heaving(ib, nx=nx, ny=ny, L=L, nsteps=10)
    wl.dt = 0.005
    out = {}
    for mode in ("graph", "eager"):
        if mode == "eager":
            monkeypatch.setenv("IBGB300_NO_GRAPH", "1")
        else:
            monkeypatch.delenv("IBGB300_NO_GRAPH", raising=False)
        prob = wl.problem()
        st = ib.initstate(prob)
        st._gamma[:] = wl.initial_gamma()
        s = ib.initsolver(prob, st, precision=precision)
        s.set_cg_options(tol=1e-10, warm_start="extrapolate")
        s.set_cg_preconditioner("schur_ref")
        s.vort2flux(st)
        for i in range(wl.nsteps):
            ib.advance_(st, s, i * wl.dt)
        it, res, r0 = s.cg_stats(wl.nsteps, start=True)
        out[mode] = (st.qty.gamma.copy(), st.qty.Fb.copy(), it, res, r0)
        s.close()
    g1, f1, it1, res1, r01 = out["graph"]
    g2, f2, it2, res2, r02 = out["eager"]
    np.testing.assert_array_equal(it1, it2)
    np.testing.assert_array_equal(g1, g2)
    np.testing.assert_array_equal(f1, f2)
    np.testing.assert_array_equal(res1, res2)
    assert np.all(res1 <= 1e-10)
