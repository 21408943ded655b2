"""Host-side logic of the Julia-API mirror and the C ABI boundary (CPU only, no GPU calls)."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_grid_sizes_and_offsets(ib, O):
    g = ib.UniformGrid(0.02, (-1.0, 3.0), (-2.0, 2.0))
    assert (g.nx, g.ny) == (200, 200)
    g2 = ib.UniformGrid(0.005, (-1.5, 3.62), (-2.56, 2.56))
    assert (g2.nx, g2.ny) == (1024, 1024)
    fluid = ib.StreamFcnFluid(ib.MultiLevel(g, 5), (1.0, 0.0), 100.0)
    d = fluid.domain
    og = O.Grid(200, 200, 5, -1.0, -2.0, 0.02)
    assert (d.nq, d.ngamma, d.L, d.R, d.B, d.T) == (og.nq, og.ngamma, og.L, og.R, og.B, og.T)
    assert ib.MultiLevel(g, 5).gridstep(3) == pytest.approx(0.08)
    # a bare UniformGrid is a 1-level MultiLevel (src/streamfcn/fluids.jl:54-57)
    assert ib.StreamFcnFluid(g, (1.0, 0.0), 100.0).domain.discrete.nlevels == 1


def test_time_range_includes_t0_like_julia(ib):
    from ibgb300.api import _time_range
    ts = _time_range(0.0, 0.004 * 499, 0.004)
    assert len(ts) == 500 and ts[0] == 0.0
    assert len(_time_range(0.0, 1.0, 0.1)) == 11
    assert len(_time_range(0.0, 0.0, 0.1)) == 1


def test_callback_callers(ib):
    from ibgb300.api import _callback_caller

    class S:
        t = 0.0
    s = S()
    calls = []
    f = _callback_caller(0.1, ib.at_indices(lambda st: calls.append(("i", st.t)), [2, 4]))
    for i in range(1, 6):
        s.t = (i - 1) * 0.1
        f(i, s)
    assert calls == [("i", pytest.approx(0.1)), ("i", pytest.approx(0.3))]
    calls.clear()
    f = _callback_caller(0.1, ib.at_times(lambda st: calls.append(st.t), [0.0, 0.11, 0.12, 0.35]))
    for i in range(1, 6):
        s.t = (i - 1) * 0.1
        f(i, s)
    # 0.0 at t=0; 0.11 and 0.12 both fall before 0.1 + dt/2 -> one call at t=0.1; 0.35 -> t=0.3
    assert calls == [0.0, pytest.approx(0.1), pytest.approx(0.3)]
    assert ib.StopIteration() == ib.StopIteration()


def test_fire_steps_schedule_matches_the_callers(ib):
    """solve_ batches the steps between firings; the schedule is the callers' own decisions."""
    from ibgb300.api import _fire_steps, _time_range
    dt = 0.1
    ts = _time_range(0.0, 1.0, dt)
    assert _fire_steps(ib.at_indices(None, [2, 4, 4, 20]), ts, dt) == {2, 4}
    assert _fire_steps(ib.at_indices(None, [4, 2]), ts, dt) == {4}
    assert _fire_steps(ib.at_times(None, [0.0, 0.11, 0.12, 0.35, 5.0]), ts, dt) == {1, 2, 4}
    assert _fire_steps(ib.each_timestep(None), ts, dt) == set(range(1, 12))


def test_circle_and_bodies(ib):
    c = ib.circle((0.0, 0.0), 0.5, 0.02)
    assert c.npoints() == int(np.floor(np.pi * 0.5 / 0.02))
    assert np.allclose(np.hypot(c.xb[:, 0], c.xb[:, 1]), 0.5)
    bg = ib.BodyGroup(c, ib.circle((1.0, 0.0), 0.25, 0.02))
    assert bg.npoints() == c.npoints() + int(np.floor(np.pi * 0.25 / 0.02))
    with pytest.raises(ValueError):
        ib.RigidBody(ib.GridFrame(), np.zeros((3, 2)), np.zeros(2))


def test_workloads(ib):
    w = ib.workloads.two_body_large()
    assert (w.nx, w.ny, w.nlevels) == (1024, 1024, 4)
    assert [b.npoints() for b in w.bodies] == [629, 201]
    assert w.cells_per_step == 4 * 1024 * 1024
    a = w.initial_gamma()
    b = w.initial_gamma()
    np.testing.assert_array_equal(a, b)
    assert a.shape == (4, 1023 * 1023) and np.all(a[1:] == 0)
    assert abs(a[0].std() / (1e-4 * 0.005 ** 2) - 1) < 0.01
    small = ib.workloads.cylinder_small()
    assert (small.nx, small.ny, small.bodies[0].npoints()) == (200, 200, 157)
    s = ib.workloads.scaled(w, 128, 128, nlevels=2)
    assert s.nx == 128 and s.ny == 128
    prob = s.problem()
    assert prob.fluid.domain.nx == 128


def test_schemes_without_solver_raise(ib):
    """SchemeCNAB and SchemeRKC have solvers; another scheme type has no state type."""
    g = ib.MultiLevel(ib.UniformGrid(0.1, (-1.0, 2.2), (-1.6, 1.6)), 2)

    class SchemeOther:
        dt = 0.01
    prob = ib.Problem(ib.StreamFcnFluid(g, (1.0, 0.0), 100.0), ib.BodyGroup(), SchemeOther())
    with pytest.raises(NotImplementedError):
        ib.initstate(prob)
    prob = ib.Problem(ib.StreamFcnFluid(g, (1.0, 0.0), 100.0), ib.BodyGroup(), ib.SchemeRKC(0.01))
    assert ib.initstate(prob).t == 0.0


def _declared_symbols():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(ib_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol(lib):
    declared = _declared_symbols()
    assert "ib_advance" in declared and "ib_create" in declared
    for name in sorted(declared):
        assert hasattr(lib, name), name
    from ibgb300 import _lib as L
    assert declared == set(L.SIGNATURES), declared ^ set(L.SIGNATURES)


def test_create_validates_arguments_without_a_gpu(lib):
    """Invalid problems are rejected on the host before any CUDA call."""
    from ibgb300 import _lib as L
    p = L.IbProblem()
    p.nx, p.ny, p.nlevels, p.h, p.dt, p.re = 30, 32, 2, 0.1, 0.01, 100.0  # nx not a multiple of 4
    h = ctypes.c_void_p()
    assert lib.ib_create(ctypes.byref(p), ctypes.byref(h)) == L.IB_ERR_INVALID
    assert b"multiples of 4" in lib.ib_last_error(None)
    p.nx = 32
    p.dt = -1.0
    assert lib.ib_create(ctypes.byref(p), ctypes.byref(h)) == L.IB_ERR_INVALID
    assert lib.ib_status_string(3) == b"infinite flux"
    assert lib.ib_advance(None, 0.0, 1.0, 0.0) == L.IB_ERR_INVALID


def test_grid_flow_of_a_translating_grid(ib):
    """base_flux! in grid coordinates: the freestream, minus a translating grid's velocity."""
    disc = ib.MultiLevel(ib.UniformGrid(0.05, (-1.0, 1.0), (-1.0, 1.0)), 2)
    lab = ib.StreamFcnFluid(disc, lambda t: (1.0 + t, 0.5), 100.0)
    assert lab.grid_flow(2.0) == (3.0, 0.5)
    frame = ib.RelativeFrame(ib.LabFrame(), r=lambda t: (0.0, 0.0), v=lambda t: (0.25, -t),
                             theta=lambda t: 0.0, omega=lambda t: 0.0)
    moving = ib.StreamFcnFluid(ib.FluidDomain(disc, frame), lambda t: (1.0 + t, 0.5), 100.0)
    assert moving.grid_flow(2.0) == (2.75, 2.5)
    prob = ib.Problem(moving, ib.BodyGroup(), ib.SchemeCNAB(0.01))
    q0 = ib.api._base_flux(prob, 2.0)
    assert np.allclose(q0[0, : moving.domain.nu], 2.75 * 0.05) and np.allclose(q0[1, moving.domain.nu:], 2.5 * 0.1)
