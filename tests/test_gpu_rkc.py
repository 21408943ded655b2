"""SchemeRKC (src/schemes.jl:3-12): the Runge-Kutta-Chebyshev scheme the reference declares
without a solver, as libibgb300 defines it (IB_SCHEME_RKC), against the oracle's restatement
(oracle.ib_oracle.RKCSolver): per-step Gamma <= 1e-10 (relative L2) and C_D / C_L <= 1e-8, the
FP64 bars; the stage count is the oracle's rule or the one given."""
import ctypes

import numpy as np
import pytest

from _util import oracle_problem, rel

pytestmark = pytest.mark.gpu


def _rkc_problem(ib, wl, stages=0):
    disc = ib.MultiLevel(ib.UniformGrid(wl.h, wl.xlims, wl.ylims), wl.nlevels)
    fs = wl.freestream
    return ib.Problem(ib.StreamFcnFluid(disc, lambda t: fs, wl.Re), ib.BodyGroup(*wl.bodies),
                      ib.SchemeRKC(wl.dt, stages=stages))


@pytest.mark.parametrize("nx,L,stages,nsteps", [(64, 2, 0, 25), (96, 3, 4, 15)])
def test_rkc_step_parity(ib, O, lib, nx, L, stages, nsteps):
    from ibgb300 import _lib as LB
    wl = ib.workloads.scaled(ib.workloads.cylinder_small(), nx, nx, nlevels=L)
    prob = _rkc_problem(ib, wl, stages)
    st = ib.initstate(prob)
    st._gamma[:] = wl.initial_gamma()
    s = ib.initsolver(prob, st)
    s.vort2flux(st)
    op = oracle_problem(O, wl, prob)
    g = op.grid
    ost = O.init_state(op)
    ost.gamma[0] = wl.initial_gamma()[0].reshape(g.gshape)
    ost.psi, ost.q = O.vort2flux(ost.gamma, g, O.lap_eigs(g))
    osol = O.RKCSolver(op, stages=stages)
    info = LB.IbInfo()
    assert lib.ib_get_info(s.handle, ctypes.byref(info)) == 0
    assert info.scheme == LB.IB_SCHEME_RKC and info.rkc_stages == osol.stages >= 2
    worst_g = worst_c = 0.0
    for i in range(nsteps):
        t = i * wl.dt
        ib.advance_(st, s, t)
        osol.advance(ost, t)
        worst_g = max(worst_g, rel(st.qty.gamma, ost.gamma.reshape(g.nlevels, -1)))
        b = st.qty.stress[0]
        worst_c = max(worst_c, abs(b.CD - ost.cd[0]) / max(1.0, abs(ost.cd[0])),
                      abs(b.CL - ost.cl[0]) / max(1.0, abs(ost.cl[0])))
    assert rel(st.qty.q, ost.q) < 1e-10
    s.close()
    print(f"RKC {nx}^2 x {L}, {osol.stages} stages: worst Gamma {worst_g:.2e}, C {worst_c:.2e}")
    assert worst_g < 1e-10 and worst_c < 1e-8, (worst_g, worst_c)


def test_rkc_limits_are_refused(ib):
    wl = ib.workloads.scaled(ib.workloads.cylinder_small(), 64, 64, nlevels=2)
    prob = _rkc_problem(ib, wl)
    st = ib.initstate(prob)
    with pytest.raises(Exception, match="FP64"):
        ib.initsolver(prob, st, precision="mixed")
