"""Shared helpers for the parity tests: build the same problem for the GPU path and the oracle."""
import ctypes

import numpy as np


def oracle_problem(O, wl, prob):
    g = O.grid_from_limits(wl.h, wl.xlims, wl.ylims, wl.nlevels)
    bodies = list(prob.bodies)
    xb = np.concatenate([b.xb for b in bodies]) if bodies else np.zeros((0, 2))
    ds = np.concatenate([b.ds for b in bodies]) if bodies else np.zeros(0)
    return O.Problem(g, wl.dt, wl.Re, xb, ds, [b.npoints() for b in bodies], freestream=wl.freestream)


def start_pair(ib, O, wl, precision="fp64"):
    """GPU state/solver and oracle state/solver from the same seeded initial condition."""
    prob = wl.problem()
    st = ib.initstate(prob)
    st._gamma[:] = wl.initial_gamma()
    solver = ib.initsolver(prob, st, precision=precision)
    solver.vort2flux(st)
    op = oracle_problem(O, wl, prob)
    g = op.grid
    ost = O.init_state(op)
    ost.gamma[0] = wl.initial_gamma()[0].reshape(g.gshape)
    ost.psi, ost.q = O.vort2flux(ost.gamma, g, O.lap_eigs(g))
    osol = O.Solver(op)
    return prob, st, solver, op, ost, osol


def rel(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


class Dev:
    """Device copies through torch (plumbing only: the compute runs in libibgb300)."""

    def __init__(self):
        import torch
        self.torch = torch

    def put(self, a):
        t = self.torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
        self.torch.cuda.synchronize()
        return t

    def empty(self, n):
        t = self.torch.zeros(int(n), dtype=self.torch.float64, device="cuda")
        self.torch.cuda.synchronize()
        return t

    @staticmethod
    def p(t):
        return ctypes.c_void_p(t.data_ptr()) if t is not None else None

    def get(self, t):
        self.torch.cuda.synchronize()
        return t.cpu().numpy()


def oracle_moving_problem(O, wl, prob, tol):
    """The oracle's MovingProblem for a workload whose bodies may move (RelativeFrame)."""
    import ibgb300 as ib
    g = O.grid_from_limits(wl.h, wl.xlims, wl.ylims, wl.nlevels)
    bodies = list(prob.bodies)

    def kin(t):
        out = []
        for b in bodies:
            f = b.frame
            if isinstance(f, ib.RelativeFrame):
                out.append((tuple(f.r(t)), tuple(f.v(t)), f.theta(t), f.omega(t)))
            else:
                out.append(((0.0, 0.0), (0.0, 0.0), 0.0, 0.0))
        return out
    ds = np.concatenate([b.ds for b in bodies])
    return O.MovingProblem(g, wl.dt, wl.Re, [b.xb for b in bodies], ds, kin, freestream=wl.freestream,
                           cg_tol=tol)
