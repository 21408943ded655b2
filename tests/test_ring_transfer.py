"""The all-levels Vort2Flux of the mixed-precision path (csrc/v2f.cu), restated in numpy and
checked against the oracle's level-by-level Vort2Flux (fluid-ops.jl:438-472).

Level l's boundary ring is get_bc! of psi_{l+1} on its quarter lines.  By linearity
psi_{l+1} = psi0_{l+1} + H(ring_{l+1}), and the harmonic part H of a ring mode k decays across
the level as sinh(th_k (m-1-J)) / (2 n sinh(th_k m)), 2 cosh th_k = 4 - 2 cos(pi (k+1)/n).  The
CUDA path keeps the first K modes per side (2 sum_{k>=K} exp(-th_k d) < 1e-17, d = the quarter
lines' distance), finds every ring first and solves all levels in one batch.  The same
construction here, in FP64, must give the oracle's psi and q to round-off.
"""
import numpy as np
import pytest

from oracle import ib_oracle as O


def decay(n, m, K):
    """g[k, J] for a side of n cells, J across m cells (closed form, exponentials only)."""
    k = np.arange(K)
    th = np.arccosh(2.0 - np.cos(np.pi * (k + 1) / n))
    J = np.arange(m - 1)
    num = np.exp(-th[:, None] * (J[None, :] + 1)) * (1 - np.exp(-2 * th[:, None] * (m - 1 - J[None, :])))
    return num / (1 - np.exp(-2 * th[:, None] * m)) / (2 * n)


def modes_kept(n, d, tol=1e-17):
    """The truncation rule of RingPlan::build (csrc/v2f.cu)."""
    th = np.arccosh(2.0 - np.cos(np.pi * np.arange(1, n) / n))
    tail = 2 * np.cumsum(np.exp(-th * d)[::-1])[::-1]
    ok = np.nonzero(tail < tol)[0]
    return int(ok[0]) if ok.size else n - 1


class Transfer:
    """ring of a level -> harmonic part of psi on the whole level, from K modes per side."""

    def __init__(self, g, K=None):
        nx, ny = g.nx, g.ny
        self.g = g
        self.Kx = modes_kept(nx, ny // 4) if K is None else K[0]
        self.Ky = modes_kept(ny, nx // 4) if K is None else K[1]
        self.Sx = 2 * np.sin(np.pi * np.outer(np.arange(1, self.Kx + 1), np.arange(1, nx)) / nx)
        self.Sy = 2 * np.sin(np.pi * np.outer(np.arange(1, self.Ky + 1), np.arange(1, ny)) / ny)
        self.gx = decay(nx, ny, self.Kx)   # [k, J]: bottom-side mode k at row J
        self.hy = decay(ny, nx, self.Ky)   # [k, I]: left-side mode k at column I

    def __call__(self, ring):
        g = self.g
        b, t = ring[g.B + 1:g.B + g.nx], ring[g.T + 1:g.T + g.nx]
        l, r = ring[g.L + 1:g.L + g.ny], ring[g.R + 1:g.R + g.ny]
        cb, ct, cl, cr = self.Sx @ b, self.Sx @ t, self.Sy @ l, self.Sy @ r
        psi = np.einsum('kI,k,kJ->JI', self.Sx, cb, self.gx) + np.einsum('kI,k,kJ->JI', self.Sx, ct, self.gx[:, ::-1])
        psi += np.einsum('kJ,k,kI->JI', self.Sy, cl, self.hy) + np.einsum('kJ,k,kI->JI', self.Sy, cr, self.hy[:, ::-1])
        return psi


def bc_field(g, ring):
    return O.apply_bc(np.zeros((g.ny - 1, g.nx - 1)), ring, 1.0, g)


def field(g, seed):
    rng = np.random.default_rng(seed)
    J, I = np.mgrid[0:g.ny - 1, 0:g.nx - 1]
    G = np.zeros((g.nlevels, g.ny - 1, g.nx - 1))
    G[0] = (np.exp(-((I - 0.45 * g.nx) ** 2 + (J - 0.5 * g.ny) ** 2) / (0.05 * g.nx) ** 2)
            - np.exp(-((I - 0.6 * g.nx) ** 2 + (J - 0.45 * g.ny) ** 2) / (0.04 * g.nx) ** 2)
            + 1e-3 * rng.standard_normal((g.ny - 1, g.nx - 1)))
    G[1] = 0.3 * np.exp(-((I - 0.3 * g.nx) ** 2 + (J - 0.5 * g.ny) ** 2) / (0.1 * g.nx) ** 2)
    return G


@pytest.mark.parametrize("nx,ny", [(256, 192), (128, 256)])
def test_truncated_transfer_is_the_harmonic_extension_on_the_quarter_lines(nx, ny):
    g = O.Grid(nx, ny, 2, 0.0, 0.0, 0.01)
    lam = O.lap_eigs(g)
    rng = np.random.default_rng(3)
    ring = rng.standard_normal(g.nbc)
    exact = O.get_bc(O.laplacian_inv(bc_field(g, ring), lam, g), g)
    tr = Transfer(g)
    full = Transfer(g, (nx - 1, ny - 1))
    assert tr.Kx < nx // 2 and tr.Ky < ny // 2
    got, ref = O.get_bc(tr(ring), g), O.get_bc(full(ring), g)
    # the kept modes reproduce the full sine expansion on the ring nodes to the last bits
    assert np.max(np.abs(got - ref)) <= 1e-15 * np.max(np.abs(ref))
    # and the full expansion is the oracle's Laplacian inverse (FFT rounding)
    assert np.max(np.abs(ref - exact)) <= 1e-12 * np.max(np.abs(exact))
    # a few modes fewer would not do
    short = O.get_bc(Transfer(g, (tr.Kx // 2, tr.Ky // 2))(ring), g)
    assert np.max(np.abs(short - ref)) > 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("nx,ny,nl", [(256, 192, 4), (192, 256, 3)])
def test_all_levels_vort2flux_matches_the_level_order(nx, ny, nl):
    g = O.Grid(nx, ny, nl, 0.0, 0.0, 0.01)
    lam = O.lap_eigs(g)
    G = field(g, nx + ny)
    Gref = G.copy()
    psi_ref, q_ref = O.vort2flux(Gref, g, lam)          # coarsifies Gref in place
    # every level's rings first: psi0 with a zero ring, then the chain through the transfer
    psi0 = O.laplacian_inv(Gref, lam, g)
    tr = Transfer(g)
    rings = np.zeros((nl, g.nbc))
    for lev in range(nl - 2, -1, -1):
        rings[lev] = O.get_bc(psi0[lev + 1], g) + O.get_bc(tr(rings[lev + 1]), g)
    # then all levels in one batch
    psi = O.laplacian_inv(Gref + np.stack([bc_field(g, r) for r in rings]), lam, g)
    q = np.stack([O.curl(psi[lev], rings[lev], g) for lev in range(nl)])
    assert np.max(np.abs(psi - psi_ref)) <= 1e-13 * np.max(np.abs(psi_ref))
    assert np.max(np.abs(q - q_ref)) <= 1e-12 * np.max(np.abs(q_ref))
