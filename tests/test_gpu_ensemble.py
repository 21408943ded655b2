"""Ensembles (include/ibgb300_ensemble.h): members of different grids and precisions advanced by
one graph launch per step, or per k steps, give exactly the steps they give alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def members(ib):
    W = ib.workloads
    return [
        (W.scaled(W.cylinder_small(), 64, 64, nlevels=2), "fp64"),
        (W.scaled(W.two_body_large(), 128, 128, nlevels=2), "mixed"),
        (W.scaled(W.cylinder_small(), 96, 80, nlevels=3), "fp64"),
        (W.scaled(W.two_body_large(), 256, 256, nlevels=3), "mixed"),
    ]


def start(ib, wl, precision):
    prob = wl.problem()
    st = ib.initstate(prob)
    st._gamma[:] = wl.initial_gamma()
    s = ib.initsolver(prob, st, precision=precision)
    # the order an ensemble gives its static members, here from the start on
    s.set_vort2flux_order("sequential")
    s.vort2flux(st)
    return prob, st, s


@pytest.mark.parametrize("per_launch", [1, 3, 4])
def test_ensemble_steps_equal_single_steps(ib, per_launch):
    """5 + 7 steps: with 3 or 4 steps per launch both the multi-step graphs (at either starting
    parity) and the single-step graphs of the remainders run."""
    n = 12
    singles = []
    for wl, prec in members(ib):
        prob, st, s = start(ib, wl, prec)
        for i in range(n):
            ib.advance_(st, s, i * 0.01)
        singles.append((st.qty.gamma.copy(), s.force_history(n)))
        s.close()
    runs = [start(ib, wl, prec) for wl, prec in members(ib)]
    ens = ib.Ensemble([r[2] for r in runs], steps_per_launch=per_launch)
    nm, kernels = ens.info()
    assert nm == 4 and kernels > 4 * 40
    ts = np.arange(n) * 0.01
    ms = ens.advance_n(ts[:5], states=[r[1] for r in runs])
    ens.advance_n(ts[5:], states=[r[1] for r in runs])
    assert ms > 0
    for (prob, st, s), (g1, (cd1, cl1)) in zip(runs, singles):
        assert st.t == ts[-1]
        np.testing.assert_array_equal(st.qty.gamma, g1)
        cd, cl = s.force_history(n)
        np.testing.assert_array_equal(cd, cd1)
        np.testing.assert_array_equal(cl, cl1)
    ens.close()
    # members continue on their own afterwards
    prob, st, s = runs[0]
    ib.advance_(st, s, n * 0.01)
    for r in runs:
        r[2].close()


def heaving(ib, f):
    W = ib.workloads
    frame = W.heave_pitch_frame(f=f, heave=0.25, pitch_deg=15.0)
    base = W.Workload("heave", 0.005, (-1.0, 2.84), (-1.28, 1.28), 2, 200.0, 0.005, 10,
                      [W.moving_plate(201, frame=frame)])
    wl = W.scaled(base, 128, 96, nlevels=2, nsteps=10)
    wl.Re, wl.dt = 200.0, 0.005
    return wl


def start_moving(ib, wl, precision):
    prob = wl.problem()
    st = ib.initstate(prob)
    st._gamma[:] = wl.initial_gamma()
    s = ib.initsolver(prob, st, precision=precision)
    s.set_cg_options(tol=1e-10, warm_start="extrapolate")
    s.set_cg_preconditioner("schur_ref")
    s.vort2flux(st)
    return prob, st, s


@pytest.mark.parametrize("per_launch", [1, 4])
def test_ensemble_with_moving_members_equals_single_steps(ib, per_launch):
    """Static and moving members (their CG loops inside the ensemble graph) give exactly the
    steps they give alone; moving members join after two steps of their own.  With 4 steps per
    launch each member's CG loops of the 4 steps run on its own branch."""
    n = 10
    cases = [("static", members(ib)[0]), ("static", members(ib)[1]),
             ("moving", (heaving(ib, 0.5), "fp64")), ("moving", (heaving(ib, 0.4), "mixed"))]
    alone = []
    for kind, (wl, prec) in cases:
        prob, st, s = (start_moving if kind == "moving" else start)(ib, wl, prec)
        for i in range(n):
            ib.advance_(st, s, i * wl.dt)
        alone.append((st.qty.gamma.copy(), s.force_history(n), s.cg_stats(n - 2)[0] if kind == "moving" else None))
        s.close()
    runs = []
    for kind, (wl, prec) in cases:
        prob, st, s = (start_moving if kind == "moving" else start)(ib, wl, prec)
        for i in range(2):
            ib.advance_(st, s, i * wl.dt)
        runs.append((kind, wl, st, s))
    dt = cases[2][1][0].dt
    assert all(r[1].dt == dt for r in runs if r[0] == "moving")
    ens = ib.Ensemble([r[3] for r in runs], steps_per_launch=per_launch)
    ts = np.arange(2, n) * dt
    ens.advance_n(ts, states=[r[2] for r in runs])
    ens.close()
    for (kind, wl, st, s), (g1, (cd1, cl1), it1) in zip(runs, alone):
        np.testing.assert_array_equal(st.qty.gamma, g1)
        cd, cl = s.force_history(n)
        np.testing.assert_array_equal(cd, cd1)
        if kind == "moving":
            np.testing.assert_array_equal(s.cg_stats(n - 2)[0], it1)
        s.close()
