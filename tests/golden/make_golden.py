"""Generate the golden fixtures in this directory from the FP64 oracle.

The reference publishes no vectors and cannot run here (Julia is not installed), so these
fixtures record the oracle's own outputs on small seeded problems.  They pin the oracle
against regressions (tests/test_golden.py re-derives them on the CPU) and give the GPU tests
a fixed target.  Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import ib_oracle as O  # noqa: E402


def cylinder_case(nx=64, ny=48, L=2, nsteps=6, seed=3):
    """Cylinder D=0.6 with points spaced ~h (like the benchmark bodies): a well-conditioned
    Schur matrix, so FP64 implementations agree to ~1e-12 on it."""
    h = 4.0 / nx
    g = O.Grid(nx, ny, L, -1.0, -0.5 * ny * h, h)
    n = 30
    t = 2 * np.pi * np.arange(n) / n
    xb = np.stack([0.6 * np.cos(t) * 0.5 + 0.3, 0.5 * 0.6 * np.sin(t)], 1)
    ds = np.full(n, np.pi * 0.6 / n)
    prob = O.Problem(g, 0.02, 100.0, xb, ds, [n])
    st = O.init_state(prob)
    rng = np.random.Generator(np.random.PCG64(seed))
    st.gamma[0] = 1e-4 * h * h * rng.standard_normal(g.gshape)
    gamma0 = st.gamma.copy()
    st.psi, st.q = O.vort2flux(st.gamma, g, O.lap_eigs(g))
    sol = O.Solver(prob)
    cd, cl = [], []
    for i in range(nsteps):
        sol.advance(st, i * prob.dt)
        cd.append(st.cd[0])
        cl.append(st.cl[0])
    return dict(nx=nx, ny=ny, L=L, h=h, x0=g.x0, y0=g.y0, dt=prob.dt, Re=prob.Re, xb=xb, ds=ds,
                seed=seed, gamma0=gamma0, cd=np.array(cd), cl=np.array(cl), gamma=st.gamma, psi=st.psi,
                q=st.q, fb=st.fb, bmat=sol.Bmat)


def kat_vectors():
    """Analytic sine-transform and Poisson known answers on a 24x20 grid."""
    g = O.Grid(24, 20, 1, 0.0, 0.0, 0.1)
    I = np.arange(1, g.nx)[None, :]
    J = np.arange(1, g.ny)[:, None]
    mode = np.sin(np.pi * 3 * I / g.nx) * np.sin(np.pi * 2 * J / g.ny)
    lam = O.lap_eigs(g)
    return dict(kat_mode=mode, kat_dst=O.dst2(mode), kat_lap_inv=O.laplacian_inv(mode, lam, g),
                kat_expected_lap_inv=mode / lam[1, 2])


if __name__ == "__main__":
    data = cylinder_case()
    data.update(kat_vectors())
    np.savez_compressed(HERE / "oracle_cylinder_64x48.npz", **data)
    print("wrote", HERE / "oracle_cylinder_64x48.npz")
