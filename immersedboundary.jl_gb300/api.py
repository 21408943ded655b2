"""Python mirror of ImmersedBoundary.jl's user API for the stream-function / CNAB path.

Same names, argument meaning and error behaviour as the reference (Julia's ``!`` suffix
becomes a trailing ``_``):

===============================  ==========================================================
reference (file:line)            here
===============================  ==========================================================
``UniformGrid`` fluids.jl:53     :class:`UniformGrid`
``MultiLevel`` fluids.jl:86      :class:`MultiLevel`
``FluidDomain`` fluids.jl:40     :class:`FluidDomain`
``GridFrame/LabFrame``           :class:`GridFrame`, :class:`LabFrame`,
  dynamics.jl:9-29                 :class:`RelativeFrame`
``StreamFcnFluid`` fluids.jl:49  :class:`StreamFcnFluid`
``RigidBody`` rigid-bodies.jl:4  :class:`RigidBody`
``BodyGroup`` bodies.jl:11       :class:`BodyGroup`
``circle`` body-tools.jl:1       :func:`circle`
``SchemeCNAB/RKC`` schemes.jl    :class:`SchemeCNAB`, :class:`SchemeRKC`
``Problem`` ImmersedBoundary:34  :class:`Problem`
``initstate/initsolver`` :51-52  :func:`initstate`, :func:`initsolver`
``advance!`` timestepping.jl:253 :func:`advance_`
``solve/solve!`` solve.jl        :func:`solve`, :func:`solve_`
``each_timestep/at_times/        :func:`each_timestep`, :func:`at_times`,
  at_indices`` solve.jl:69-91      :func:`at_indices`, :class:`StopIteration`
``StateResult`` solve.jl:145     :class:`StateResult`
===============================  ==========================================================

The state lives on the GPU once a solver exists; ``state.qty`` fields are read back
lazily (only when a callback or the caller touches them).
"""
from __future__ import annotations

import ctypes as C
import os
import math
from dataclasses import dataclass
from typing import Callable, Sequence

import numpy as np

from . import _lib

__all__ = [
    "UniformGrid", "MultiLevel", "FluidDomain", "GridFrame", "LabFrame", "RelativeFrame",
    "StreamFcnFluid", "RigidBody", "BodyGroup", "circle", "npoints", "SchemeCNAB", "SchemeRKC",
    "Problem", "State", "StreamFcnQuantities", "BodyStress", "Solver", "initstate", "initsolver",
    "advance_", "solve", "solve_", "each_timestep", "at_times", "at_indices", "StopIteration",
    "StateResult", "timestep", "gridstep", "Ensemble",
]


# ---------------------------------------------------------------------------------------------
# frames (src/dynamics.jl:9-29)
# ---------------------------------------------------------------------------------------------
class GridFrame:
    """Bodies fixed in the grid frame (``GridFrame``, dynamics.jl:12)."""

    def __eq__(self, other):
        return isinstance(other, GridFrame)

    def __hash__(self):
        return hash("GridFrame")


class LabFrame:
    """The lab frame (``LabFrame``, dynamics.jl:13); the default fluid frame."""

    def __eq__(self, other):
        return isinstance(other, LabFrame)

    def __hash__(self):
        return hash("LabFrame")


@dataclass
class RelativeFrame:
    """``RelativeFrame{F}(base, r, v, θ, Ω)`` (dynamics.jl:23-29): moving-body kinematics."""

    base: object
    r: Callable[[float], Sequence[float]]
    v: Callable[[float], Sequence[float]]
    theta: Callable[[float], float]
    omega: Callable[[float], float]


# ---------------------------------------------------------------------------------------------
# grids (src/fluids/fluids.jl)
# ---------------------------------------------------------------------------------------------
def _range_len(a: float, b: float, h: float) -> int:
    """Length of Julia's ``a:h:b`` (rounded like Julia's exact-rational range length)."""
    r = (b - a) / h
    n = round(r)
    if abs(r - n) > 1e-9 * max(1.0, abs(r)):
        n = math.floor(r)
    return int(n) + 1


class UniformGrid:
    """``UniformGrid(h, (x0, x1), (y0, y1))`` (fluids.jl:53-56): ``xs = x0:h:x1``, ``ys = y0:h:y1``."""

    def __init__(self, h: float, xlims: Sequence[float], ylims: Sequence[float]):
        self.h = float(h)
        nxp = _range_len(float(xlims[0]), float(xlims[1]), self.h)
        nyp = _range_len(float(ylims[0]), float(ylims[1]), self.h)
        self.xs = float(xlims[0]) + self.h * np.arange(nxp)
        self.ys = float(ylims[0]) + self.h * np.arange(nyp)

    @property
    def nx(self) -> int:
        return len(self.xs) - 1

    @property
    def ny(self) -> int:
        return len(self.ys) - 1

    def xycoords(self):
        return self.xs, self.ys

    def gridstep(self) -> float:
        return self.h


class MultiLevel:
    """``MultiLevel(base, nlevels)`` (fluids.jl:86-95): nested levels, each doubling extent and h."""

    def __init__(self, base: UniformGrid, nlevels: int):
        if nlevels < 1:
            raise ValueError("nlevels must be >= 1")
        self.base = base
        self.nlevels = int(nlevels)

    def baselevel(self) -> UniformGrid:
        return self.base

    def gridstep(self, lev: int) -> float:
        """``gridstep(domain, lev) = h * 2^(lev-1)`` (fluids.jl:102)."""
        return self.base.h * 2.0 ** (lev - 1)


def gridstep(grid, lev: int | None = None) -> float:
    return grid.gridstep() if lev is None else grid.gridstep(lev)


class FluidDomain:
    """``FluidDomain(discrete, frame=LabFrame())`` (fluids.jl:40-45)."""

    def __init__(self, discrete, frame=None):
        self.discrete = discrete
        self.frame = frame if frame is not None else LabFrame()


class StreamFcnGrid:
    """``StreamFcnGrid`` sizes and BC offsets (src/streamfcn/fluids.jl:3-45)."""

    def __init__(self, domain: FluidDomain):
        disc = domain.discrete
        if isinstance(disc, UniformGrid):
            disc = MultiLevel(disc, 1)
        self.discrete: MultiLevel = disc
        self.frame = domain.frame
        base = disc.base
        nx, ny = base.nx, base.ny
        self.nx, self.ny = nx, ny
        self.nu = (nx + 1) * ny
        self.nq = self.nu + nx * (ny + 1)
        self.ngamma = (nx - 1) * (ny - 1)
        self.L, self.R, self.B, self.T = 0, ny + 1, 2 * (ny + 1), 2 * (ny + 1) + nx + 1


class StreamFcnFluid:
    """``StreamFcnFluid(domain, freestream, Re)`` (src/streamfcn/fluids.jl:49-58).

    ``domain`` is a :class:`UniformGrid`, :class:`MultiLevel` or :class:`FluidDomain`;
    ``freestream`` maps ``t -> (u, v)`` (a constant pair is accepted too).
    """

    def __init__(self, domain, freestream, Re: float):
        if not isinstance(domain, FluidDomain):
            domain = FluidDomain(domain)
        self.domain = StreamFcnGrid(domain)
        self._fs = freestream
        self.Re = float(Re)

    def freestream(self, t: float):
        f = self._fs
        u, v = (f(t) if callable(f) else f)
        return float(u), float(v)

    def grid_flow(self, t: float):
        """The uniform flow the base flux carries, in grid coordinates (``base_flux!``,
        fluid-ops.jl:403-419).  LabFrame (or GridFrame) fluid: the freestream.  A fluid whose
        grid translates with a ``RelativeFrame(LabFrame(), r, v, θ, Ω)`` (the reference's
        "TODO: moving grid", :419): the freestream seen from the grid, U(t) - v(t); the grid
        frame must not rotate (θ = Ω = 0), since a rotating grid would add fictitious terms the
        scheme does not have."""
        u, v = self.freestream(t)
        fr = self.domain.frame
        if isinstance(fr, RelativeFrame):
            if fr.theta(t) != 0.0 or fr.omega(t) != 0.0:
                raise NotImplementedError("a rotating grid frame is not supported (theta and Omega must be 0)")
            gv = fr.v(t)
            return u - float(gv[0]), v - float(gv[1])
        return u, v


# ---------------------------------------------------------------------------------------------
# bodies (src/bodies)
# ---------------------------------------------------------------------------------------------
class RigidBody:
    """``RigidBody(frame, xb::Matrix (n x 2), ds::Vector)`` (rigid-bodies.jl:4-10)."""

    def __init__(self, frame, xb, ds):
        self.frame = frame
        self.xb = np.array(xb, dtype=np.float64).reshape(-1, 2)
        self.ds = np.array(ds, dtype=np.float64).reshape(-1)
        if self.ds.shape[0] != self.xb.shape[0]:
            raise ValueError("xb and ds have different point counts")

    def npoints(self) -> int:
        return self.xb.shape[0]


def npoints(b) -> int:
    return b.npoints()


class BodyGroup(list):
    """``BodyGroup(bodies...)`` (bodies.jl:11-21)."""

    def __init__(self, *bodies):
        if len(bodies) == 1 and not isinstance(bodies[0], RigidBody):
            bodies = tuple(bodies[0])
        super().__init__(bodies)

    def npoints(self) -> int:
        return int(sum(b.npoints() for b in self))


def circle(center, r: float, h: float, frame=None) -> RigidBody:
    """``circle((x, y), r, h; frame=GridFrame())`` (body-tools.jl:1-10): n = floor(pi r/h) points."""
    x, y = center
    n = int(math.floor(math.pi * r / h))
    t = 2 * math.pi / n * np.arange(n)
    xb = np.stack([x + r * np.cos(t), y + r * np.sin(t)], axis=1)
    ds = math.hypot(xb[1, 0] - xb[0, 0], xb[1, 1] - xb[0, 1])
    return RigidBody(frame if frame is not None else GridFrame(), xb, np.full(n, ds))


# ---------------------------------------------------------------------------------------------
# schemes and problem (src/schemes.jl, src/ImmersedBoundary.jl)
# ---------------------------------------------------------------------------------------------
class SchemeCNAB:
    """``SchemeCNAB(dt)``: 2-step Crank-Nicolson / Adams-Bashforth, beta = [1.5, -0.5] (schemes.jl:19-26)."""

    def __init__(self, dt: float):
        self.beta = (1.5, -0.5)
        self.dt = float(dt)


class SchemeRKC:
    """``SchemeRKC(dt)`` (schemes.jl:3-12), which the reference declares without a solver.  Here
    the s-stage second-order Runge-Kutta-Chebyshev method (damping 2/13) on the explicit
    vorticity transport dGamma/dt = nu lap(Gamma) + N(Gamma), followed by the immersed-boundary
    projection; ``stages`` = 0 picks the fewest stages whose stability interval covers
    1.5 x dt x 8 / (Re h^2).  FP64, bodies fixed in the grid."""

    def __init__(self, dt: float, stages: int = 0):
        self.dt = float(dt)
        self.stages = int(stages)


def timestep(x) -> float:
    return x.scheme.dt if isinstance(x, Problem) else x.dt


class Problem:
    """``Problem(fluid, bodies, scheme)`` (src/ImmersedBoundary.jl:34-38)."""

    def __init__(self, fluid: StreamFcnFluid, bodies: BodyGroup, scheme):
        self.fluid = fluid
        self.bodies = bodies if isinstance(bodies, BodyGroup) else BodyGroup(bodies)
        self.scheme = scheme


# ---------------------------------------------------------------------------------------------
# state (src/streamfcn/states.jl, src/streamfcn/cnab/states.jl)
# ---------------------------------------------------------------------------------------------
@dataclass
class BodyStress:
    """``BodyStress(fb, CD, CL)`` (states.jl:3-7): surface stress and force coefficients."""

    fb: np.ndarray
    CD: float
    CL: float


def _base_flux(prob: Problem, t: float) -> np.ndarray:
    """``base_flux!`` (fluid-ops.jl:403-417) as a host array (nq x nlevels, column-major)."""
    d = prob.fluid.domain
    L = d.discrete.nlevels
    u, v = prob.fluid.grid_flow(t)
    q0 = np.empty((L, d.nq))
    for lev in range(1, L + 1):
        hc = d.discrete.gridstep(lev)
        q0[lev - 1, : d.nu] = u * hc
        q0[lev - 1, d.nu:] = v * hc
    return q0


class StreamFcnQuantities:
    """``StreamFcnQuantities`` (states.jl:9-41).  Arrays are (nlevels, n) C-order, i.e. the
    transpose view of the reference's (n x nlevels) column-major matrices (same memory)."""

    def __init__(self, state: "State"):
        self._state = state

    def _pull(self):
        self._state._pull()
        return self._state

    @property
    def gamma(self) -> np.ndarray:
        return self._pull()._gamma

    @property
    def q(self) -> np.ndarray:
        return self._pull()._q

    @property
    def psi(self) -> np.ndarray:
        return self._pull()._psi

    @property
    def q0(self) -> np.ndarray:
        return _base_flux(self._state.prob, self._state.t)

    @property
    def Fb(self) -> np.ndarray:
        return self._pull()._fb

    @property
    def stress(self) -> list:
        return self._state._stress_list()

    @property
    def points(self):
        """``BodyGroupPoints`` (body-points.jl:6-10): (positions, velocities), each (nb, 2)."""
        s = self._state._solver
        if s is None:
            xb = np.concatenate([b.xb for b in self._state.prob.bodies]) if len(self._state.prob.bodies) else np.zeros((0, 2))
            return xb, np.zeros_like(xb)
        return s.body_points()

    # Julia field names
    Γ = gamma
    ψ = psi


class State:
    """``CNAB.State`` (cnab/states.jl:1-16): ``qty``, ``nonlin`` (2 matrices) and ``t``."""

    def __init__(self, prob: Problem, t: float = 0.0):
        d = prob.fluid.domain
        L = d.discrete.nlevels
        self.prob = prob
        self.t = float(t)
        self._gamma = np.zeros((L, d.ngamma))
        self._psi = np.zeros((L, d.ngamma))
        self._q = np.zeros((L, d.nq))
        self._fb = np.zeros(2 * prob.bodies.npoints())
        self._nonlin = [np.zeros((L, d.ngamma)), np.zeros((L, d.ngamma))]
        self._solver: Solver | None = None
        self._stale = False
        self.qty = StreamFcnQuantities(self)

    @property
    def nonlin(self) -> list:
        self._pull()
        return self._nonlin

    def _pull(self):
        s = self._solver
        if self._stale and s is not None:
            s._get_state(self)
            self._stale = False

    def _stress_list(self) -> list:
        s = self._solver
        nb_list = [b.npoints() for b in self.prob.bodies]
        if s is None:
            return [BodyStress(np.zeros((n, 2)), 0.0, 0.0) for n in nb_list]
        cd, cl, fbs = s.stress()
        out, i = [], 0
        for k, n in enumerate(nb_list):
            blk = fbs[2 * i: 2 * i + 2 * n].reshape(2, n).T.copy()
            out.append(BodyStress(blk, float(cd[k]), float(cl[k])))
            i += n
        return out


def initstate(prob: Problem, t: float = 0.0) -> State:
    """``initstate(prob, t)`` (src/ImmersedBoundary.jl:51)."""
    if not isinstance(prob.scheme, (SchemeCNAB, SchemeRKC)):
        raise NotImplementedError(f"no state type for scheme {type(prob.scheme).__name__}")
    return State(prob, t)


# ---------------------------------------------------------------------------------------------
# solver (the GPU handle)
# ---------------------------------------------------------------------------------------------
class Solver:
    """``CNAB.Solver`` (cnab/timestepping.jl:173-249) backed by a libibgb300 handle.

    ``precision``: ``"fp64"`` (every sine transform in FP64, the reference's arithmetic),
    ``"mixed"`` (FP32 sine transforms refined with float-float residuals, ``refine_sweeps`` sweeps per
    Poisson solve: 1 or 2 everywhere, or 0 = the library default of 2 with 1 for the Vort2Flux
    solves of the third and coarser levels; state, stencils and the nonlinear term in float-float
    arithmetic; Schur solve and forces FP64), or ``"mixed_tc"`` (the same solve with every sine
    transform a BF16x3 split-precision GEMM against the sine matrix on the tensor cores; both
    axes a multiple of 128 cells).
    """

    def __init__(self, prob: Problem, state: State, device: int = 0, history_capacity: int = 4096,
                 precision: str = "fp64", refine_sweeps: int = 0):
        if not isinstance(prob.scheme, (SchemeCNAB, SchemeRKC)):
            raise NotImplementedError(f"no solver for scheme {type(prob.scheme).__name__}")
        for b in prob.bodies:
            if not isinstance(b.frame, (GridFrame, RelativeFrame)):
                raise NotImplementedError(f"unsupported body frame {type(b.frame).__name__}")
        # bodies in a RelativeFrame move rigidly (their xb are body-frame coordinates)
        self.moving = any(isinstance(b.frame, RelativeFrame) for b in prob.bodies)
        fr = prob.fluid.domain.frame
        if not isinstance(fr, (LabFrame, GridFrame)) and not (isinstance(fr, RelativeFrame)
                                                             and isinstance(fr.base, LabFrame)):
            raise NotImplementedError("the fluid frame must be LabFrame, GridFrame or a RelativeFrame of LabFrame")
        self.lib = _lib.load()
        self.prob = prob
        d = prob.fluid.domain
        base = d.discrete.base
        self.L = d.discrete.nlevels
        self.d = d
        bodies = prob.bodies
        npts = np.array([b.npoints() for b in bodies], dtype=np.int32)
        xb = np.concatenate([b.xb for b in bodies], axis=0) if len(bodies) else np.zeros((0, 2))
        ds = np.concatenate([b.ds for b in bodies]) if len(bodies) else np.zeros(0)
        self._xb = np.ascontiguousarray(xb.T).reshape(-1)  # column-major nb x 2
        self._ds = np.ascontiguousarray(ds, dtype=np.float64)
        self._npts = npts
        self.nbodies = len(bodies)
        self.nb = int(npts.sum())
        p = _lib.IbProblem()
        p.nx, p.ny, p.nlevels = base.nx, base.ny, self.L
        p.x0, p.y0, p.h = float(base.xs[0]), float(base.ys[0]), base.h
        p.dt = prob.scheme.dt
        if isinstance(prob.scheme, SchemeRKC):
            p.beta0, p.beta1 = 1.5, -0.5
            p.scheme = _lib.IB_SCHEME_RKC
            p.rkc_stages = prob.scheme.stages
        else:
            p.beta0, p.beta1 = prob.scheme.beta
            p.scheme = _lib.IB_SCHEME_CNAB
        p.re = prob.fluid.Re
        p.nbodies = self.nbodies
        p.body_npoints = _lib.iptr(self._npts) if self.nbodies else None
        p.xb = _lib.dptr(self._xb) if self.nb else None
        p.ds = _lib.dptr(self._ds) if self.nb else None
        p.motion = _lib.IB_MOTION_PRESCRIBED if self.moving else _lib.IB_MOTION_STATIC
        if precision not in _lib.PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(_lib.PRECISIONS)}")
        self.precision = precision
        p.precision = _lib.PRECISIONS[precision]
        p.device = device
        p.history_capacity = history_capacity
        p.refine_sweeps = refine_sweeps
        h = C.c_void_p()
        _lib.check(self.lib, None, self.lib.ib_create(C.byref(p), C.byref(h)))
        self.handle = h
        self._set_state(state)
        state._solver = self
        self._bound_state = state

    def close(self):
        if getattr(self, "handle", None):
            self.lib.ib_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, status):
        return _lib.check(self.lib, self.handle, status)

    def _set_state(self, st: State):
        self._check(self.lib.ib_set_state(
            self.handle, _lib.dptr(st._gamma), _lib.dptr(st._q), _lib.dptr(st._psi),
            _lib.dptr(st._nonlin[0]), _lib.dptr(st._nonlin[1]),
            _lib.dptr(st._fb) if st._fb.size else None, st.t))

    def _get_state(self, st: State):
        t = C.c_double()
        self._check(self.lib.ib_get_state(
            self.handle, _lib.dptr(st._gamma), _lib.dptr(st._q), _lib.dptr(st._psi),
            _lib.dptr(st._nonlin[0]), _lib.dptr(st._nonlin[1]),
            _lib.dptr(st._fb) if st._fb.size else None, C.byref(t)))

    def save_checkpoint(self, path) -> None:
        """Write the state a restart needs (Gamma, q, psi, nonlin, Fb, t, step count) to a
        checkpoint file (layout in include/ibgb300.h, ``ib_checkpoint_save``)."""
        self._check(self.lib.ib_checkpoint_save(self.handle, os.fsencode(str(path))))

    def load_checkpoint(self, path, state: "State | None" = None) -> None:
        """Restore a checkpoint into this handle (same grid, levels, points and motion); the
        bound state's host copies refresh from the device when next read."""
        self._check(self.lib.ib_checkpoint_load(self.handle, os.fsencode(str(path))))
        st = state if state is not None else getattr(self, "_bound_state", None)
        if st is not None:
            t = C.c_double()
            self._check(self.lib.ib_get_state(self.handle, None, None, None, None, None, None, C.byref(t)))
            st.t = t.value
            st._stale = True

    _FORMS = ("stockham", "warp", "tensor")

    def autotune(self) -> dict:
        """The setup-time autotuner's measurements: device ms of its timed unit per candidate
        ``"<form>/<order>[/y8]"`` (form: stockham, warp or tensor; order: levels or sequential;
        ``/y8``: the warp y pass compiled for 8 resident blocks per SM) and the candidate in
        effect (``None`` if the tuner did not run)."""
        ms = np.zeros(12)
        ch = C.c_int32()
        self._check(self.lib.ib_get_autotune(self.handle, _lib.dptr(ms), C.byref(ch)))

        def name(i):
            return (f"{self._FORMS[i // 4]}/{'levels' if (i // 2) % 2 else 'sequential'}"
                    + ("/y8" if i % 2 else ""))
        out = {name(i): float(ms[i]) for i in range(12) if ms[i] > 0}
        c = ch.value
        return {"ms": out, "chosen": None if c < 0 else name(c)}

    def stress(self):
        nbd = max(self.nbodies, 1)
        cd = np.zeros(nbd)
        cl = np.zeros(nbd)
        fbs = np.zeros(max(2 * self.nb, 1))
        self._check(self.lib.ib_get_stress(self.handle, _lib.dptr(cd), _lib.dptr(cl), _lib.dptr(fbs)))
        return cd, cl, fbs

    def force_history(self, count: int):
        nbd = max(self.nbodies, 1)
        cd = np.zeros((count, nbd))
        cl = np.zeros((count, nbd))
        self._check(self.lib.ib_get_force_history(self.handle, count, _lib.dptr(cd), _lib.dptr(cl)))
        return cd[:, : self.nbodies], cl[:, : self.nbodies]

    def kinematics(self, t: float) -> np.ndarray:
        """Per body (r0x, r0y, v0x, v0y, θ, Ω) at t from the RelativeFrame closures
        (src/dynamics.jl:23-29); bodies fixed in the grid get the identity motion."""
        k = np.zeros((self.nbodies, 6))
        for i, b in enumerate(self.prob.bodies):
            f = b.frame
            if isinstance(f, RelativeFrame):
                r, v = f.r(t), f.v(t)
                k[i] = (r[0], r[1], v[0], v[1], f.theta(t), f.omega(t))
        return k

    def set_cg_options(self, tol: float = 1e-10, maxiter: int = 5000, warm_start: str = "previous"):
        """CG tolerance (||r|| / ||rhs||), cap and warm start ("previous", "extrapolate", "zero" or
        "learned": the trained network of ``learn_init`` / ``learn_train``)."""
        mode = {"previous": _lib.IB_WARM_PREVIOUS, "extrapolate": _lib.IB_WARM_EXTRAPOLATE,
                "zero": _lib.IB_WARM_ZERO, "learned": _lib.IB_WARM_LEARNED}[warm_start]
        self._check(self.lib.ib_set_cg_options(self.handle, float(tol), int(maxiter), mode))

    def set_cg_preconditioner(self, mode: str = "schur_ref", refresh_steps: int = 0):
        """``"none"`` (plain CG, the reference's) or ``"schur_ref"``: PCG with the inverse Schur
        matrix of a reference configuration, re-assembled every ``refresh_steps`` steps or, with 0,
        once the extra iterations since the last assembly have cost as much time as an assembly."""
        m = {"none": _lib.IB_PC_NONE, "schur_ref": _lib.IB_PC_SCHUR_REF}[mode]
        self._check(self.lib.ib_set_cg_preconditioner(self.handle, m, int(refresh_steps)))

    def set_vort2flux_order(self, order: str = "auto"):
        """Mixed precision: ``"levels"`` (every level's boundary ring first, then all levels in
        one batch), ``"sequential"`` (the reference's coarse-to-fine order) or ``"auto"`` (levels
        up to 2^20 cells per level where the grid allows it).  FP64 solvers keep the reference
        order."""
        m = {"auto": _lib.IB_V2F_AUTO, "levels": _lib.IB_V2F_LEVELS, "sequential": _lib.IB_V2F_SEQUENTIAL}[order]
        self._check(self.lib.ib_set_vort2flux_order(self.handle, m))

    def cg_preconditioner_stats(self, seconds: bool = False):
        """(assemblies, step of the last one[, its duration in seconds])."""
        n, last, sec = C.c_int32(), C.c_int64(), C.c_double()
        self._check(self.lib.ib_get_cg_preconditioner_stats(self.handle, C.byref(n), C.byref(last), C.byref(sec)))
        return (n.value, last.value, sec.value) if seconds else (n.value, last.value)

    def cg_stats(self, count: int, start: bool = False):
        """Iterations and final relative residuals of the last `count` CG solves (and, with
        ``start``, the initial relative residuals of their warm starts)."""
        it = np.zeros(count, dtype=np.int32)
        res = np.zeros(count)
        self._check(self.lib.ib_get_cg_stats(self.handle, count, _lib.iptr(it), _lib.dptr(res)))
        if not start:
            return it, res
        r0 = np.zeros(count)
        self._check(self.lib.ib_get_cg_start_residuals(self.handle, count, _lib.dptr(r0)))
        return it, res, r0

    # learned warm start (include/ibgb300_learn.h)
    def learn_init(self, hidden: int = 256, layers: int = 3, capacity: int = 4096, seed: int = 0):
        self._check(self.lib.ib_learn_init(self.handle, int(hidden), int(layers), int(capacity), int(seed)))

    def learn_collect(self, on: bool = True):
        self._check(self.lib.ib_learn_collect(self.handle, 1 if on else 0))

    def learn_samples(self) -> int:
        n = C.c_int32()
        self._check(self.lib.ib_learn_sample_count(self.handle, C.byref(n)))
        return n.value

    def learn_train(self, epochs: int = 200, batch: int = 64, lr: float = 1e-3, seed: int = 0) -> float:
        loss = C.c_double()
        self._check(self.lib.ib_learn_train(self.handle, int(epochs), int(batch), float(lr), int(seed),
                                            C.byref(loss)))
        return loss.value

    def learn_validation(self):
        """(blend, held-out error relative to plain extrapolation) of the last training."""
        b, r = C.c_double(), C.c_double()
        self._check(self.lib.ib_learn_validation(self.handle, C.byref(b), C.byref(r)))
        return b.value, r.value

    def learn_set_blend(self, blend: float):
        """Weight of the network's correction in the warm start (0: plain extrapolation)."""
        self._check(self.lib.ib_learn_set_blend(self.handle, float(blend)))

    def learn_export(self) -> np.ndarray:
        """The trained network with its normalisation and blend (``ib_learn_export``)."""
        dims = self.learn_layout()
        npar = C.c_int64()
        self._check(self.lib.ib_learn_param_count(self.handle, C.byref(npar)))
        n = int(npar.value) + 2 * dims[0] + 2 * dims[-1] + 1
        buf = np.zeros(n, dtype=np.float32)
        self._check(self.lib.ib_learn_export(self.handle, _lib.fptr(buf), n))
        return buf

    def learn_import(self, buf: np.ndarray):
        """Load a network exported from a handle of the same layout; marks it trained."""
        b = np.ascontiguousarray(buf, dtype=np.float32)
        self._check(self.lib.ib_learn_import(self.handle, _lib.fptr(b), int(b.size)))

    def learn_layout(self):
        nl = C.c_int32()
        dims = np.zeros(16, dtype=np.int32)
        self._check(self.lib.ib_learn_layout(self.handle, C.byref(nl), _lib.iptr(dims), 16))
        return [int(d) for d in dims[: nl.value + 1]]

    def learn_params(self, params: np.ndarray | None = None) -> np.ndarray:
        """Get (or, given ``params``, set) the FP32 parameter vector."""
        n = C.c_int64()
        self._check(self.lib.ib_learn_param_count(self.handle, C.byref(n)))
        if params is not None:
            p = np.ascontiguousarray(params, dtype=np.float32)
            assert p.size == n.value
            self._check(self.lib.ib_learn_set_params(self.handle, _lib.fptr(p)))
            return p
        out = np.zeros(n.value, dtype=np.float32)
        self._check(self.lib.ib_learn_get_params(self.handle, _lib.fptr(out)))
        return out

    def learn_gradients(self, x: np.ndarray, y: np.ndarray):
        """(loss, gradient) of the raw network on rows x, targets y (no normalisation)."""
        n = C.c_int64()
        self._check(self.lib.ib_learn_param_count(self.handle, C.byref(n)))
        xa = np.ascontiguousarray(x, dtype=np.float32)
        ya = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(n.value, dtype=np.float32)
        loss = C.c_double()
        self._check(self.lib.ib_learn_gradients(self.handle, int(xa.shape[0]), _lib.fptr(xa), _lib.fptr(ya),
                                                _lib.fptr(g), C.byref(loss)))
        return loss.value, g

    def body_points(self):
        xb = np.zeros(2 * max(self.nb, 1))
        vb = np.zeros(2 * max(self.nb, 1))
        self._check(self.lib.ib_get_body_points(self.handle, _lib.dptr(xb), _lib.dptr(vb)))
        n = self.nb
        return xb[: 2 * n].reshape(2, n).T.copy(), vb[: 2 * n].reshape(2, n).T.copy()

    def advance(self, state: State, t: float):
        u, v = self.prob.fluid.grid_flow(t)
        if self.moving:
            kin = np.ascontiguousarray(self.kinematics(t).reshape(-1))
            self._check(self.lib.ib_advance_kin(self.handle, float(t), u, v, _lib.dptr(kin)))
        else:
            self._check(self.lib.ib_advance(self.handle, float(t), u, v))
        state.t = float(t)
        state._stale = True

    def _after_ensemble(self, t, state: State | None):
        st = state if state is not None else getattr(self, "_bound_state", None)
        if st is not None and t is not None:
            st.t = t
            st._stale = True

    def vort2flux(self, state: State):
        """``solver.vort2flux!(state.qty)`` (fluid-ops.jl:438): psi and q from Gamma, on the GPU."""
        self._check(self.lib.ib_vort2flux(self.handle))
        state._stale = True

    def advance_n(self, state: State, ts: Sequence[float]):
        ts = np.ascontiguousarray(np.asarray(ts, dtype=np.float64))
        if ts.size == 0:
            return
        uv = np.ascontiguousarray(np.array([self.prob.fluid.grid_flow(t) for t in ts], dtype=np.float64).reshape(-1))
        if self.moving:
            kin = np.ascontiguousarray(np.concatenate([self.kinematics(t).reshape(-1) for t in ts]))
            self._check(self.lib.ib_advance_n_kin(self.handle, int(ts.size), _lib.dptr(ts), _lib.dptr(uv),
                                                  _lib.dptr(kin)))
        else:
            self._check(self.lib.ib_advance_n(self.handle, int(ts.size), _lib.dptr(ts), _lib.dptr(uv)))
        state.t = float(ts[-1])
        state._stale = True


def initsolver(prob: Problem, state: State, **kw) -> Solver:
    """``initsolver(prob, state)`` (src/ImmersedBoundary.jl:52)."""
    s = Solver(prob, state, **kw)
    return s


def advance_(state: State, solver: Solver, t: float):
    """``advance!(state, solver, t)`` (cnab/timestepping.jl:253-290)."""
    solver.advance(state, t)


class Ensemble:
    """Independent simulations advanced together by one graph launch per step
    (include/ibgb300_ensemble.h; no reference counterpart).  Moving members join after their
    first two steps.  Members keep their own state; ``state`` objects are refreshed lazily like
    after ``advance_``."""

    def __init__(self, solvers: Sequence[Solver], steps_per_launch: int = 1):
        self.solvers = list(solvers)
        self.lib = self.solvers[0].lib
        arr = (C.c_void_p * len(self.solvers))(*[s.handle for s in self.solvers])
        h = C.c_void_p()
        st = self.lib.ib_ensemble_create(arr, len(self.solvers), C.byref(h))
        if st != _lib.IB_OK:
            raise _lib.IBError(st, (self.lib.ib_ensemble_last_error(None) or b"").decode())
        self.handle = h
        if steps_per_launch != 1:
            self.set_steps_per_launch(steps_per_launch)

    def _check(self, st):
        if st != _lib.IB_OK:
            raise _lib.IBError(st, (self.lib.ib_ensemble_last_error(self.handle) or b"").decode())

    def info(self):
        n, k = C.c_int32(), C.c_int32()
        self._check(self.lib.ib_ensemble_info(self.handle, C.byref(n), C.byref(k)))
        return n.value, k.value

    def set_steps_per_launch(self, k: int):
        """Carry ``k`` consecutive steps of every member per graph launch (1..8): within a
        launch a member goes on with its next step without waiting for the slowest member.
        Results are bitwise those of one step per launch."""
        self._check(self.lib.ib_ensemble_set_steps_per_launch(self.handle, int(k)))

    def advance_n(self, ts, uv=None, states: Sequence[State] | None = None) -> float:
        """Advance every member through the times ``ts``: [nsteps] (the same times for every
        member) or [nsteps][members] (each member's own times, e.g. t0 + k dt of its scheme);
        freestream per member and step in ``uv`` [nsteps][members][2] (default: each member's
        problem freestream at its time).  Returns the device milliseconds."""
        ts = np.asarray(ts, dtype=np.float64)
        n = len(self.solvers)
        if ts.ndim == 1:
            ts = np.repeat(ts[:, None], n, axis=1)
        ts = np.ascontiguousarray(ts)
        if uv is None:
            uv = np.array([[s.prob.fluid.grid_flow(float(ts[k, i])) for i, s in enumerate(self.solvers)]
                           for k in range(ts.shape[0])], dtype=np.float64)
        uv = np.ascontiguousarray(uv, dtype=np.float64)
        ms = C.c_double()
        movers = [i for i, s in enumerate(self.solvers) if s.moving]
        if movers:
            kin = np.ascontiguousarray(np.concatenate(
                [np.concatenate([self.solvers[i].kinematics(float(ts[k, i])).reshape(-1) for i in movers])
                 for k in range(ts.shape[0])]))
            self._check(self.lib.ib_ensemble_advance_n_kin(self.handle, len(ts), _lib.dptr(ts), _lib.dptr(uv),
                                                           _lib.dptr(kin), C.byref(ms)))
        else:
            self._check(self.lib.ib_ensemble_advance_n(self.handle, len(ts), _lib.dptr(ts), _lib.dptr(uv),
                                                       C.byref(ms)))
        for k, s in enumerate(self.solvers):
            s._after_ensemble(float(ts[-1, k]) if len(ts) else None, states[k] if states else None)
        return ms.value

    def close(self):
        if self.handle:
            self.lib.ib_ensemble_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------------------------
# driver and callbacks (src/solve.jl)
# ---------------------------------------------------------------------------------------------
class StopIteration:  # noqa: A001 - mirrors the reference's StopIteration() sentinel
    """Returned by a callback to stop :func:`solve` (solve.jl:1-6)."""

    def __eq__(self, other):
        return isinstance(other, StopIteration)

    def __hash__(self):
        return hash("StopIteration")


class _AllTimesteps:
    pass


@dataclass
class _TimestepIndices:
    i: Sequence[int]


@dataclass
class _TimestepTimes:
    t: Sequence[float]


@dataclass
class StateCallback:
    """``StateCallback(f, timesteps, ret)`` (solve.jl:52-58)."""

    f: Callable
    timesteps: object
    ret: type = object


def each_timestep(f, ret=object) -> StateCallback:
    """``each_timestep(f, [ret])`` (solve.jl:69)."""
    return StateCallback(f, _AllTimesteps(), ret)


def at_times(f, t, ret=object) -> StateCallback:
    """``at_times(f, t, [ret])`` (solve.jl:80)."""
    return StateCallback(f, _TimestepTimes(list(t)), ret)


def at_indices(f, i, ret=object) -> StateCallback:
    """``at_indices(f, i, [ret])`` (solve.jl:91)."""
    return StateCallback(f, _TimestepIndices(list(i)), ret)


class StateResult(list):
    """``StateResult{T}`` (solve.jl:145-157): results with their times in ``.t``."""

    def __init__(self):
        super().__init__()
        self.t: list[float] = []


def _callback_caller(dt: float, cb: StateCallback):
    """``_callback_caller`` (solve.jl:106-134).

    The reference dispatches ``at_times`` callers on ``dt::Float64`` but ``solve!`` passes the
    time range when building result pushers (solve.jl:178,196), a MethodError; here ``dt`` is
    always the step, so ``at_times`` also works in ``save``.
    """
    ts = cb.timesteps
    if isinstance(ts, _AllTimesteps):
        return lambda i, state: cb.f(state)
    if isinstance(ts, _TimestepIndices):
        it = list(ts.i)
        pos = [0]

        def call_idx(i, state):
            if pos[0] < len(it) and it[pos[0]] == i:
                pos[0] += 1
                return cb.f(state)
            return None
        return call_idx
    it = list(ts.t)
    pos = [0]
    half = dt / 2

    def call_t(i, state):
        call = False
        while pos[0] < len(it) and it[pos[0]] < state.t + half:
            pos[0] += 1
            call = True
        return cb.f(state) if call else None
    return call_t


def _time_range(t0: float, tf: float, dt: float) -> np.ndarray:
    n = int(math.floor((tf - t0) / dt + 1e-10)) + 1
    return t0 + dt * np.arange(max(n, 0))


def solve_(state: State, prob: Problem, tlims, save=(), call=(), solver: Solver | None = None):
    """``solve!(state, problem, (t0, tf); save, call)`` (solve.jl:188-215).

    ``advance!`` runs at every t in ``t0:dt:tf`` including t0.  With no callbacks the steps
    are issued as one batch of captured-graph replays.
    """
    solver = solver or initsolver(prob, state)
    dt = timestep(prob)
    t0, tf = tlims
    ts = _time_range(float(t0), float(tf), dt)
    callers = [_callback_caller(dt, cb) for cb in call]
    results = [StateResult() for _ in save]

    def pusher(cb, res):
        inner = _callback_caller(dt, StateCallback(lambda s: cb.f(s), cb.timesteps))

        def p(i, s):
            u = inner(i, s)
            if u is not None:
                res.append(u)
                res.t.append(s.t)
        return p

    pushers = [pusher(cb, r) for cb, r in zip(save, results)]
    # Steps at which some callback fires, known before stepping: every caller's decision is a
    # function of the step index and time alone.  The steps in between run as batches of
    # captured-graph replays without a host round trip.
    fire = sorted(set().union(*(_fire_steps(cb, ts, dt) for cb in (*save, *call))))
    done = 0
    for k in fire:
        for c0 in range(done, k, 1024):
            solver.advance_n(state, ts[c0:min(k, c0 + 1024)])
        done = k
        for p in pushers:
            p(k, state)
        stop = False
        for f in callers:
            stop |= f(k, state) == StopIteration()
        if stop:
            return results
    for c0 in range(done, len(ts), 1024):
        solver.advance_n(state, ts[c0:c0 + 1024])
    return results


def _fire_steps(cb: StateCallback, ts: np.ndarray, dt: float) -> set:
    """The 1-based step indices at which ``cb``'s caller calls it over the time range ``ts``."""
    caller = _callback_caller(dt, StateCallback(lambda s: True, cb.timesteps))

    class _At:
        t = 0.0
    at = _At()
    out = set()
    for i, t in enumerate(ts, start=1):
        at.t = float(t)
        if caller(i, at) is not None:
            out.add(i)
    return out


def solve(prob: Problem, tlims, save=(), call=(), **kw):
    """``solve(problem, (t0, tf); save, call)`` (solve.jl:231)."""
    return solve_(initstate(prob, tlims[0]), prob, tlims, save=save, call=call, **kw)
