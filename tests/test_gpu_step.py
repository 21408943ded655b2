"""Step-level parity of the CUDA advance! against the FP64 oracle, through the C ABI.

Tolerances (the bar for the FP64 path): per-step vorticity relative L2 <= 1e-10 and
C_L / C_D <= 1e-8 (relative to max(1, |C|)), over the whole run; bitwise run-to-run.
"""
import os

import numpy as np
import pytest

from _util import rel, start_pair

pytestmark = pytest.mark.gpu

G_TOL = 1e-10
C_TOL = 1e-8


def cerr(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(1.0, np.abs(b))))


def run_parity(ib, O, wl, nsteps, check_every=1, precision="fp64", gtol=G_TOL, ftol=1e-8):
    prob, st, solver, op, ost, osol = start_pair(ib, O, wl, precision)
    g = op.grid
    worst_g = worst_c = 0.0
    for i in range(nsteps):
        t = i * wl.dt
        ib.advance_(st, solver, t)
        osol.advance(ost, t)
        stress = st.qty.stress
        cd = [s.CD for s in stress]
        cl = [s.CL for s in stress]
        worst_c = max(worst_c, cerr(cd, ost.cd), cerr(cl, ost.cl))
        if (i + 1) % check_every == 0 or i == nsteps - 1:
            worst_g = max(worst_g, rel(st.qty.gamma, ost.gamma.reshape(g.nlevels, -1)))
    # full state at the end
    assert rel(st.qty.psi, ost.psi.reshape(g.nlevels, -1)) < gtol
    assert rel(st.qty.q, ost.q) < gtol
    assert rel(st.qty.Fb, ost.fb) < ftol
    assert rel(st.nonlin[1], ost.nonlin[1].reshape(g.nlevels, -1)) < gtol
    for k, s in enumerate(st.qty.stress):
        assert rel(s.fb, ost.stress[k]) < ftol
    solver.close()
    return worst_g, worst_c


def test_step_parity_small_cylinder(ib, O):
    wl = ib.workloads.scaled(ib.workloads.cylinder_small(), 64, 48, nlevels=3)
    wg, wc = run_parity(ib, O, wl, 30)
    assert wg < G_TOL and wc < C_TOL, (wg, wc)


def test_step_parity_two_bodies(ib, O):
    wl = ib.workloads.scaled(ib.workloads.two_body_large(), 128, 128, nlevels=2)
    wg, wc = run_parity(ib, O, wl, 15)
    assert wg < G_TOL and wc < C_TOL, (wg, wc)


def test_step_parity_cylinder_small_full_size(ib, O):
    """The 200x200, 5-level, 157-point cylinder at Re=100 (first 100 of its 500 steps)."""
    wl = ib.workloads.cylinder_small(nsteps=100)
    wg, wc = run_parity(ib, O, wl, 100, check_every=10)
    assert wg < G_TOL and wc < C_TOL, (wg, wc)


def test_no_body_freestream_stays_zero(ib):
    grid = ib.MultiLevel(ib.UniformGrid(0.05, (-1.0, 2.2), (-1.6, 1.6)), 2)
    prob = ib.Problem(ib.StreamFcnFluid(grid, (1.0, 0.0), 100.0), ib.BodyGroup(), ib.SchemeCNAB(0.01))
    st = ib.initstate(prob)
    solver = ib.initsolver(prob, st)
    for i in range(3):
        ib.advance_(st, solver, i * 0.01)
    assert np.all(st.qty.gamma == 0.0) and np.all(st.qty.q == 0.0)
    solver.close()


def test_bitwise_deterministic_and_graph_equals_eager(ib):
    wl = ib.workloads.scaled(ib.workloads.two_body_large(), 96, 96, nlevels=3)
    outs = []
    for no_graph in ("0", "0", "1"):
        os.environ["IBGB300_NO_GRAPH"] = no_graph
        try:
            prob = wl.problem()
            st = ib.initstate(prob)
            st._gamma[:] = wl.initial_gamma()
            s = ib.initsolver(prob, st)
            s.vort2flux(st)
            for i in range(8):
                ib.advance_(st, s, i * wl.dt)
            outs.append((st.qty.gamma.copy(), st.qty.Fb.copy()))
            s.close()
        finally:
            os.environ.pop("IBGB300_NO_GRAPH", None)
    for a, b in outs[1:]:
        np.testing.assert_array_equal(a, outs[0][0])
        np.testing.assert_array_equal(b, outs[0][1])


def test_advance_n_and_solve_callbacks_match_single_steps(ib):
    wl = ib.workloads.scaled(ib.workloads.cylinder_small(), 64, 64, nlevels=2)
    prob = wl.problem()
    # single steps with a per-step callback
    cds = ib.solve(prob, (0.0, 9 * wl.dt), save=(ib.each_timestep(lambda s: s.qty.stress[0].CD),))[0]
    assert len(cds) == 10 and cds.t[0] == 0.0
    # batched graph replays, then the device force history
    st = ib.initstate(prob)
    s = ib.initsolver(prob, st)
    ib.solve_(st, prob, (0.0, 9 * wl.dt), solver=s)
    cd_hist, _ = s.force_history(10)
    np.testing.assert_array_equal(cd_hist[:, 0], np.array(cds))
    assert st.t == pytest.approx(9 * wl.dt)
    s.close()


def test_stop_iteration_and_at_indices(ib):
    wl = ib.workloads.scaled(ib.workloads.cylinder_small(), 64, 64, nlevels=2)
    prob = wl.problem()
    seen = []

    def stopper(s):
        seen.append(s.t)
        return ib.StopIteration() if len(seen) == 4 else None
    res = ib.solve(prob, (0.0, 20 * wl.dt), save=(ib.at_indices(lambda s: s.t, [2, 3]),),
                   call=(ib.each_timestep(stopper),))
    assert len(seen) == 4
    assert list(res[0]) == pytest.approx([wl.dt, 2 * wl.dt])


def test_sparse_callbacks_run_batched_and_match_single_steps(ib):
    """at_indices / at_times callbacks: the steps between firings run as graph-replay batches
    and the samples equal those of a per-step run."""
    wl = ib.workloads.scaled(ib.workloads.cylinder_small(), 64, 64, nlevels=2)
    prob = wl.problem()
    every = ib.solve(prob, (0.0, 29 * wl.dt), save=(ib.each_timestep(lambda s: s.qty.gamma.copy()),))[0]
    idx = [1, 7, 20, 30]
    times = [0.0, 4.6 * wl.dt, 12.2 * wl.dt]
    res = ib.solve(prob, (0.0, 29 * wl.dt),
                   save=(ib.at_indices(lambda s: s.qty.gamma.copy(), idx),
                         ib.at_times(lambda s: s.qty.gamma.copy(), times)))
    assert len(res[0]) == 4 and len(res[1]) == 3
    for got, i in zip(res[0], idx):
        np.testing.assert_array_equal(got, every[i - 1])
    for got, i in zip(res[1], [1, 6, 13]):
        np.testing.assert_array_equal(got, every[i - 1])
    assert res[1].t == pytest.approx([0.0, 5 * wl.dt, 12 * wl.dt])


def test_errors_are_reported_not_faulted(ib):
    """A body too close to the edge and a non-finite state come back as status codes."""
    grid = ib.MultiLevel(ib.UniformGrid(0.05, (-1.0, 2.2), (-1.6, 1.6)), 2)
    fluid = ib.StreamFcnFluid(grid, (1.0, 0.0), 100.0)
    edge = ib.RigidBody(ib.GridFrame(), np.array([[-0.98, 0.0], [-0.9, 0.0]]), np.array([0.05, 0.05]))
    prob = ib.Problem(fluid, ib.BodyGroup(edge), ib.SchemeCNAB(0.01))
    with pytest.raises(ib.IBError) as e:
        ib.initsolver(prob, ib.initstate(prob))
    assert e.value.status == 4
    body = ib.circle((0.5, 0.0), 0.4, 0.05)
    prob = ib.Problem(fluid, ib.BodyGroup(body), ib.SchemeCNAB(0.01))
    st = ib.initstate(prob)
    st._q[0, 10] = np.nan
    s = ib.initsolver(prob, st)
    with pytest.raises(ib.IBError) as e:
        ib.advance_(st, s, 0.0)
    assert e.value.status == 3
    s.close()


# Mixed precision (FP32 sine transforms + two float-float residual refinement sweeps per solve): the bar is
# C_L / C_D within 1e-6 of the FP64 oracle; vorticity is checked at 1e-8 relative L2.
M_GTOL = 1e-8
M_CTOL = 1e-6


def test_mixed_parity_two_bodies(ib, O):
    wl = ib.workloads.scaled(ib.workloads.two_body_large(), 128, 128, nlevels=3)
    wg, wc = run_parity(ib, O, wl, 40, precision="mixed", gtol=M_GTOL, ftol=1e-6)
    assert wg < M_GTOL and wc < M_CTOL, (wg, wc)


def test_mixed_parity_cylinder_small_full_size(ib, O):
    wl = ib.workloads.cylinder_small(nsteps=100)
    wg, wc = run_parity(ib, O, wl, 100, check_every=10, precision="mixed", gtol=M_GTOL, ftol=1e-6)
    assert wg < M_GTOL and wc < M_CTOL, (wg, wc)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-9)])
def test_warp_and_stockham_transforms_agree(ib, monkeypatch, precision, tol):
    """The warp-per-line passes (both axes 64 P cells; IBGB300_DST=warp) and the shared-memory
    Stockham passes (IBGB300_DST=stockham) give the same steps to round-off."""
    wl = ib.workloads.scaled(ib.workloads.two_body_large(), 256, 256, nlevels=3)
    out = {}
    for mode in ("warp", "stockham"):
        monkeypatch.setenv("IBGB300_DST", mode)
        prob = wl.problem()
        st = ib.initstate(prob)
        st._gamma[:] = wl.initial_gamma()
        s = ib.initsolver(prob, st, precision=precision)
        s.vort2flux(st)
        cds = []
        for i in range(10):
            ib.advance_(st, s, i * wl.dt)
            cds.append([b.CD for b in st.qty.stress])
        out[mode] = (st.qty.gamma.copy(), np.array(cds))
        s.close()
    assert rel(out["warp"][0], out["stockham"][0]) < tol
    assert np.max(np.abs(out["warp"][1] - out["stockham"][1])) < tol * 100


def test_two_warp_lines_agree_with_one_warp_lines(ib, monkeypatch):
    """Lines transformed by two warps (IBGB300_LINE_LANES=64) and by one warp give the same
    mixed-precision steps to round-off."""
    wl = ib.workloads.scaled(ib.workloads.two_body_large(), 256, 256, nlevels=3)
    out = {}
    for lanes in ("32", "64"):
        monkeypatch.setenv("IBGB300_LINE_LANES", lanes)
        prob = wl.problem()
        st = ib.initstate(prob)
        st._gamma[:] = wl.initial_gamma()
        s = ib.initsolver(prob, st, precision="mixed")
        s.vort2flux(st)
        for i in range(10):
            ib.advance_(st, s, i * wl.dt)
        out[lanes] = st.qty.gamma.copy()
        s.close()
    assert rel(out["64"], out["32"]) < 1e-9


@pytest.mark.parametrize("nx,ny,nl", [(256, 192, 4), (192, 256, 3), (128, 128, 2)])
def test_levels_vort2flux_matches_level_by_level(ib, monkeypatch, nx, ny, nl):
    """Mixed-precision Vort2Flux with every level's boundary ring found first (harmonic ring
    transfer) and the levels solved as one batch, against the reference's level-by-level order
    (IBGB300_V2F=sequential) in mixed precision and in FP64: the same fields to round-off."""
    wl = ib.workloads.scaled(ib.workloads.cylinder_small(), nx, ny, nlevels=nl)
    out = {}
    for mode, prec in (("levels", "mixed"), ("sequential", "mixed"), ("sequential", "fp64")):
        monkeypatch.setenv("IBGB300_V2F", mode)
        prob = wl.problem()
        st = ib.initstate(prob)
        st._gamma[:] = wl.initial_gamma()
        s = ib.initsolver(prob, st, precision=prec)
        s.vort2flux(st)
        first = (st.qty.psi.copy(), st.qty.q.copy())
        cds = []
        for i in range(12):
            ib.advance_(st, s, i * wl.dt)
            cds.append([b.CD for b in st.qty.stress] + [b.CL for b in st.qty.stress])
        out[mode, prec] = first + (st.qty.psi.copy(), st.qty.q.copy(), st.qty.gamma.copy(), np.array(cds))
        s.close()
    lv, sq, fp = out["levels", "mixed"], out["sequential", "mixed"], out["sequential", "fp64"]
    for k in range(5):  # psi, q of the initial field; psi, q, Gamma after 12 steps
        assert rel(lv[k], fp[k]) < 1e-10, (k, rel(lv[k], fp[k]), rel(sq[k], fp[k]))
    assert np.max(np.abs(lv[5] - fp[5]) / np.maximum(1.0, np.abs(fp[5]))) < 1e-8


def test_vort2flux_order_setter(ib):
    """ib_set_vort2flux_order switches a mixed solver between the two Vort2Flux orders (the step
    graphs are captured again); both give the FP64 steps to round-off.  The all-levels order
    needs one-warp line passes on both axes."""
    W = ib.workloads
    wl = W.scaled(W.two_body_large(), 256, 256, nlevels=3)
    out = {}
    for prec, orders in (("fp64", ("auto",)), ("mixed", ("sequential", "levels", "auto"))):
        prob = wl.problem()
        st = ib.initstate(prob)
        st._gamma[:] = wl.initial_gamma()
        s = ib.initsolver(prob, st, precision=prec)
        s.vort2flux(st)
        for k in range(9):
            s.set_vort2flux_order(orders[k % len(orders)])
            ib.advance_(st, s, k * wl.dt)
        out[prec] = st.qty.gamma.copy()
        s.close()
    assert rel(out["mixed"], out["fp64"]) < 1e-10
    wl2 = W.scaled(W.cylinder_small(), 96, 80, nlevels=2)
    prob = wl2.problem()
    st = ib.initstate(prob)
    s = ib.initsolver(prob, st, precision="mixed")
    with pytest.raises(ib.IBError):
        s.set_vort2flux_order("levels")
    s.set_vort2flux_order("sequential")
    s.close()
