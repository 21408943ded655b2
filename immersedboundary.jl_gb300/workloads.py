"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference ships no datasets or benchmark inputs; these builders create the problems
the benchmark configurations describe (grids, bodies, Reynolds numbers, time steps) and the
seeded initial vorticity noise (NumPy PCG64), identical for the GPU path and the oracle.

* ``cylinder_small``   200x200, h=0.02, 5 levels, cylinder D=1 (157 points), Re=100, dt=0.004
* ``two_body_large``   1024x1024, h=0.005, 4 levels, cylinder D=1 at (0,0.8) (629 points) and
                       a flat plate, chord 1 at 20 deg, centred at (0,-0.8) (201 points),
                       Re=200, dt=0.001
* ``four_cylinders``   2048x2048, h=0.0025, 5 levels, four cylinders D=0.5 on a 2x2 lattice of
                       spacing 1.5 (629 points each), Re=150, dt=0.0005
* ``heaving_plate``    768x512, h=0.005, 4 levels, flat plate chord 1 (201 points) heaving
                       y = 0.5 sin(2 pi f t) and pitching 30 deg sin(2 pi f t + pi/2) about its
                       quarter chord, f = 0.2, Re=1000, dt=0.0005 (at dt=0.001 the explicit
                       advection of the CNAB step grows by ~4x per step from step 5)
* ``ensemble``         independent members: finest grid drawn from {128x128, 256x256,
                       384x256, 512x512}, h = 4/nx, 3-5 levels, an ellipse of chord 1 with aspect
                       ratio U[0.1, 1] at U[0, 40] deg (points ~h apart), Re log-uniform in
                       [50, 500], dt = 0.2 h; every other member pitches about mid-chord at
                       15 deg amplitude and frequency U[0.1, 0.3] (moving=True)
* ``scaled(...)``      the same bodies on coarser grids, for tests
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .api import (BodyGroup, GridFrame, MultiLevel, Problem, RelativeFrame, RigidBody, SchemeCNAB,
                  StreamFcnFluid, UniformGrid)

NOISE = 1e-4


def cylinder(center, D: float, n: int, frame=None) -> RigidBody:
    """n equally spaced points on a circle of diameter D (ds = pi D / n)."""
    t = 2 * math.pi * np.arange(n) / n
    r = D / 2
    xb = np.stack([center[0] + r * np.cos(t), center[1] + r * np.sin(t)], axis=1)
    return RigidBody(frame or GridFrame(), xb, np.full(n, math.pi * D / n))


def flat_plate(center, chord: float, aoa_deg: float, n: int, frame=None) -> RigidBody:
    """n equally spaced points on a plate; positive angle of attack raises the leading edge."""
    a = math.radians(aoa_deg)
    s = np.linspace(-chord / 2, chord / 2, n)
    xb = np.stack([center[0] + s * math.cos(a), center[1] - s * math.sin(a)], axis=1)
    return RigidBody(frame or GridFrame(), xb, np.full(n, chord / (n - 1)))


@dataclass
class Workload:
    name: str
    h: float
    xlims: tuple
    ylims: tuple
    nlevels: int
    Re: float
    dt: float
    nsteps: int
    bodies: list = field(default_factory=list)
    freestream: tuple = (1.0, 0.0)
    seed: int = 0

    def problem(self) -> Problem:
        grid = MultiLevel(UniformGrid(self.h, self.xlims, self.ylims), self.nlevels)
        fs = self.freestream
        fluid = StreamFcnFluid(grid, lambda t: fs, self.Re)
        return Problem(fluid, BodyGroup(*self.bodies), SchemeCNAB(self.dt))

    @property
    def nx(self) -> int:
        return int(round((self.xlims[1] - self.xlims[0]) / self.h))

    @property
    def ny(self) -> int:
        return int(round((self.ylims[1] - self.ylims[0]) / self.h))

    @property
    def cells_per_step(self) -> int:
        """Unit of work: L * nx * ny cells advanced by one step (every level does equal work)."""
        return self.nlevels * self.nx * self.ny

    def initial_gamma(self) -> np.ndarray:
        """(nlevels, (nx-1)(ny-1)) circulation: seeded N(0,1) vorticity noise of amplitude 1e-4
        on the finest level (Gamma = omega h^2), zero elsewhere."""
        ng = (self.nx - 1) * (self.ny - 1)
        g = np.zeros((self.nlevels, ng))
        rng = np.random.Generator(np.random.PCG64(self.seed))
        g[0] = NOISE * self.h * self.h * rng.standard_normal(ng)
        return g


def cylinder_small(nsteps: int = 500, seed: int = 0) -> Workload:
    return Workload("cylinder_small", 0.02, (-1.0, 3.0), (-2.0, 2.0), 5, 100.0, 0.004, nsteps,
                    [cylinder((0.0, 0.0), 1.0, 157)], seed=seed)


def two_body_large(nsteps: int = 2000, seed: int = 0) -> Workload:
    return Workload("two_body_large", 0.005, (-1.5, 3.62), (-2.56, 2.56), 4, 200.0, 0.001, nsteps,
                    [cylinder((0.0, 0.8), 1.0, 629), flat_plate((0.0, -0.8), 1.0, 20.0, 201)], seed=seed)


def four_cylinders(nsteps: int = 2000, seed: int = 0) -> Workload:
    cyl = [cylinder((x, y), 0.5, 629) for y in (-0.75, 0.75) for x in (-0.75, 0.75)]
    return Workload("four_cylinders", 0.0025, (-2.0, 3.12), (-2.56, 2.56), 5, 150.0, 0.0005, nsteps, cyl,
                    seed=seed)


def ellipse(center, chord: float, aspect: float, angle_deg: float, h: float, frame=None) -> RigidBody:
    """Points ~h apart (equal arc length) on an ellipse of major axis `chord` and minor axis
    aspect*chord, rotated by angle_deg (leading edge up for positive angles)."""
    a, b = chord / 2, aspect * chord / 2
    th = np.linspace(0, 2 * math.pi, 4097)
    x, y = a * np.cos(th), b * np.sin(th)
    s = np.concatenate([[0.0], np.cumsum(np.hypot(np.diff(x), np.diff(y)))])
    n = max(8, int(round(s[-1] / h)))
    sk = np.arange(n) * s[-1] / n
    xs, ys = np.interp(sk, s, x), np.interp(sk, s, y)
    c, sn = math.cos(math.radians(angle_deg)), math.sin(math.radians(angle_deg))
    xb = np.stack([center[0] + c * xs + sn * ys, center[1] - sn * xs + c * ys], axis=1)
    return RigidBody(frame or GridFrame(), xb, np.full(n, s[-1] / n))


def pitch_frame(f: float, amp_deg: float = 15.0) -> RelativeFrame:
    """Pitching about the frame origin: theta = A sin(2 pi f t)."""
    w = 2 * math.pi * f
    a = math.radians(amp_deg)
    return RelativeFrame(GridFrame(), r=lambda t: (0.0, 0.0), v=lambda t: (0.0, 0.0),
                         theta=lambda t: a * math.sin(w * t), omega=lambda t: a * w * math.cos(w * t))


def ensemble(n: int = 96, nsteps: int = 1000, seed: int = 0, moving: bool = False) -> list[Workload]:
    rng = np.random.default_rng(seed)
    grids = [(128, 128), (256, 256), (384, 256), (512, 512)]
    out = []
    for k in range(n):
        nx, ny = grids[rng.integers(len(grids))]
        h = 4.0 / nx
        L = int(rng.integers(3, 6))
        aspect = float(rng.uniform(0.1, 1.0))
        angle = float(rng.uniform(0.0, 40.0))
        re = float(np.exp(rng.uniform(np.log(50.0), np.log(500.0))))
        f = float(rng.uniform(0.1, 0.3))
        frame = pitch_frame(f) if (moving and k % 2 == 1) else None
        body = ellipse((0.0, 0.0), 1.0, aspect, angle, h, frame=frame)
        out.append(Workload(f"member{k}", h, (-1.5, 2.5), (-ny * h / 2, ny * h / 2), L, re, 0.2 * h, nsteps,
                            [body], seed=seed + k))
    return out


def heave_pitch_frame(f: float = 0.2, heave: float = 0.5, pitch_deg: float = 30.0) -> RelativeFrame:
    """RelativeFrame of a plate heaving y = A sin(2 pi f t) and pitching about the frame origin
    theta = P sin(2 pi f t + pi/2)."""
    w = 2 * math.pi * f
    p = math.radians(pitch_deg)
    return RelativeFrame(GridFrame(),
                         r=lambda t: (0.0, heave * math.sin(w * t)),
                         v=lambda t: (0.0, heave * w * math.cos(w * t)),
                         theta=lambda t: p * math.sin(w * t + math.pi / 2),
                         omega=lambda t: p * w * math.cos(w * t + math.pi / 2))


def moving_plate(n: int, chord: float = 1.0, frame=None) -> RigidBody:
    """Body-frame plate of n points with the pitch axis (frame origin) at the quarter chord."""
    s = np.linspace(-0.25 * chord, 0.75 * chord, n)
    xb = np.stack([s, np.zeros(n)], axis=1)
    return RigidBody(frame or heave_pitch_frame(), xb, np.full(n, chord / (n - 1)))


def heaving_plate(nsteps: int = 4000, f: float = 0.2, seed: int = 0, dt: float = 0.0005) -> Workload:
    return Workload("heaving_plate", 0.005, (-1.0, 2.84), (-1.28, 1.28), 4, 1000.0, dt, nsteps,
                    [moving_plate(201, frame=heave_pitch_frame(f))], seed=seed)


def scaled(base: Workload, nx: int, ny: int | None = None, nlevels: int | None = None,
           nsteps: int | None = None) -> Workload:
    """The same domain and bodies on an nx x ny finest grid (body points re-spaced to ~h)."""
    ny = ny or int(round(nx * (base.ylims[1] - base.ylims[0]) / (base.xlims[1] - base.xlims[0])))
    h = (base.xlims[1] - base.xlims[0]) / nx
    ylims = (base.ylims[0], base.ylims[0] + ny * h)
    bodies = []
    for b in base.bodies:
        # keep each body's shape, with about one point per cell
        xb = b.xb
        per = np.sum(np.hypot(*np.diff(np.vstack([xb, xb[:1]]), axis=0).T))
        closed = np.hypot(*(xb[-1] - xb[0])) < 2 * b.ds[0]
        length = per if closed else per - np.hypot(*(xb[-1] - xb[0]))
        n = max(8, int(round(length / h)))
        idx = np.linspace(0, xb.shape[0] - (0 if closed else 1), n, endpoint=not closed)
        x = np.interp(idx, np.arange(xb.shape[0] + (1 if closed else 0)),
                      np.append(xb[:, 0], xb[0, 0]) if closed else xb[:, 0])
        y = np.interp(idx, np.arange(xb.shape[0] + (1 if closed else 0)),
                      np.append(xb[:, 1], xb[0, 1]) if closed else xb[:, 1])
        bodies.append(RigidBody(b.frame, np.stack([x, y], 1), np.full(n, length / (n if closed else n - 1))))
    return Workload(f"{base.name}_{nx}x{ny}", h, base.xlims, ylims, nlevels or base.nlevels, base.Re,
                    base.dt * (h / base.h), nsteps or base.nsteps, bodies, base.freestream, base.seed)
