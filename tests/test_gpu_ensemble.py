"""Ensembles (include/ibgb300_ensemble.h): members of different grids and precisions advanced by
one graph launch per step give exactly the steps they give alone."""
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
    s.vort2flux(st)
    return prob, st, s


def test_ensemble_steps_equal_single_steps(ib):
    n = 12
    singles = []
    for wl, prec in members(ib):
        prob, st, s = start(ib, wl, prec)
        for i in range(n):
            ib.advance_(st, s, i * 0.01)
        singles.append((st.qty.gamma.copy(), s.force_history(n)))
        s.close()
    runs = [start(ib, wl, prec) for wl, prec in members(ib)]
    ens = ib.Ensemble([r[2] for r in runs])
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


def test_ensemble_rejects_moving_members(ib):
    wl = ib.workloads.scaled(ib.workloads.heaving_plate(nsteps=2), 128, 96, nlevels=2)
    prob = wl.problem()
    st = ib.initstate(prob)
    s = ib.initsolver(prob, st)
    with pytest.raises(ib.IBError):
        ib.Ensemble([s])
    s.close()
