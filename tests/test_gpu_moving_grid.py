"""A grid that translates with the body (base_flux! for a moving grid; the reference leaves it as
a TODO at src/streamfcn/fluid-ops.jl:419): the fluid's frame is a RelativeFrame of the lab
frame, so the base flux carries the freestream seen from the grid, U(t) - v_grid(t).

* A cylinder towed through fluid at rest with velocity v(t), solved in a grid that moves with
  it, equals the same cylinder fixed in a lab-frame grid with freestream -v(t) (same bits).
* Against the oracle's moving-grid base flux: the FP64 bars (Gamma 1e-10, C 1e-8).
"""
import math

import numpy as np
import pytest

from _util import rel

pytestmark = pytest.mark.gpu


def _vel(t):
    return (-1.0 - 0.3 * math.sin(2.0 * t), 0.1 * math.cos(3.0 * t))


def _problem(ib, wl, moving_grid: bool):
    disc = ib.MultiLevel(ib.UniformGrid(wl.h, wl.xlims, wl.ylims), wl.nlevels)
    if moving_grid:
        frame = ib.RelativeFrame(ib.LabFrame(), r=lambda t: (0.0, 0.0), v=_vel, theta=lambda t: 0.0,
                                 omega=lambda t: 0.0)
        fluid = ib.StreamFcnFluid(ib.FluidDomain(disc, frame), lambda t: (0.0, 0.0), wl.Re)
    else:
        fluid = ib.StreamFcnFluid(disc, lambda t: (-_vel(t)[0], -_vel(t)[1]), wl.Re)
    return ib.Problem(fluid, ib.BodyGroup(*wl.bodies), ib.SchemeCNAB(wl.dt))


def test_towed_cylinder_in_a_moving_grid_equals_the_lab_frame_problem(ib, O):
    wl = ib.workloads.scaled(ib.workloads.cylinder_small(), 64, 64, nlevels=2)
    runs = []
    for mg in (True, False):
        prob = _problem(ib, wl, mg)
        st = ib.initstate(prob)
        st._gamma[:] = wl.initial_gamma()
        s = ib.initsolver(prob, st)
        s.vort2flux(st)
        for i in range(6):
            ib.advance_(st, s, i * wl.dt)
        runs.append((st.qty.gamma.copy(), st.qty.Fb.copy(), st.qty.stress[0].CD))
        s.close()
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])
    # the oracle with the grid's velocity subtracted in its base flux
    prob = _problem(ib, wl, True)
    g = O.grid_from_limits(wl.h, wl.xlims, wl.ylims, wl.nlevels)
    xb = np.concatenate([b.xb for b in prob.bodies])
    ds = np.concatenate([b.ds for b in prob.bodies])
    op = O.Problem(g, wl.dt, wl.Re, xb, ds, [b.npoints() for b in prob.bodies], freestream=(0.0, 0.0),
                   grid_velocity=_vel)
    ost = O.init_state(op)
    ost.gamma[0] = wl.initial_gamma()[0].reshape(g.gshape)
    ost.psi, ost.q = O.vort2flux(ost.gamma, g, O.lap_eigs(g))
    osol = O.Solver(op)
    for i in range(6):
        osol.advance(ost, i * wl.dt)
    assert rel(runs[0][0], ost.gamma.reshape(g.nlevels, -1)) < 1e-10
    assert abs(runs[0][2] - ost.cd[0]) / max(1.0, abs(ost.cd[0])) < 1e-8


def test_rotating_grid_is_refused(ib):
    wl = ib.workloads.scaled(ib.workloads.cylinder_small(), 64, 64, nlevels=2)
    disc = ib.MultiLevel(ib.UniformGrid(wl.h, wl.xlims, wl.ylims), wl.nlevels)
    frame = ib.RelativeFrame(ib.LabFrame(), r=lambda t: (0.0, 0.0), v=lambda t: (0.0, 0.0),
                             theta=lambda t: 0.1 * t, omega=lambda t: 0.1)
    fluid = ib.StreamFcnFluid(ib.FluidDomain(disc, frame), (1.0, 0.0), wl.Re)
    with pytest.raises(NotImplementedError):
        fluid.grid_flow(0.5)
