"""FP64 CPU oracle for the Colonius-Taira IBPM / CNAB step of ImmersedBoundary.jl.

TEST INFRASTRUCTURE ONLY.  This module is the checker: the parity tests, the
``smoke()`` entry point and the ``cpu_baseline`` / ``--impl reference`` legs of
``bench.py`` are the only callers.  The product path (``libibgb300.so`` and the
Python host mirror) never imports it.

It restates, function by function, the reference's Julia code for the
stream-function / CNAB path (file:line cited on each function, paths relative
to the ImmersedBoundary.jl project root) in NumPy/SciPy FP64.  The 2-D DST-I is
``scipy.fft.dstn(type=1)``, which uses the same unnormalised convention as the
FFTW ``RODFT00`` plan the reference builds (FFTW 3.3.10 via FFTW.jl 1.5.0,
``src/streamfcn/fluid-ops.jl:25``).  The dense Schur inverse is
``numpy.linalg.inv`` standing in for Julia's ``inv`` (LAPACK getrf/getri,
``src/streamfcn/cnab/ops.jl:96``).

Parity unpinned: the reference ships no tests, fixtures or golden vectors and
Julia is not available to run it, so this restatement is pinned only against
known-answer identities derived from the reference's own formulas (DST-I
involution, curl/rot Laplacian identity, CN eigen-multipliers, E/E^T
adjointness, delta-function moments, freestream invariance).

Array layout: every per-level array uses the reference's column-major layout,
held in NumPy as C-order arrays indexed ``[..., j, i]`` (``i`` fastest), so a
level's flat vector is ``a.reshape(-1)`` and equals the Julia vector.

* circulation / streamfunction: ``(..., ny-1, nx-1)``
* x-flux ``qx``: ``(..., ny, nx+1)``; y-flux ``qy``: ``(..., ny+1, nx)``
* boundary ring ``bc``: ``(..., 2(nx+1)+2(ny+1))`` with offsets L/R/B/T.
* body forces ``Fb``: ``[fx_1..fx_nb, fy_1..fy_nb]``.

Leading ``...`` axes are batch axes (used to assemble Schur columns in bulk).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
from scipy import fft as sfft

#: scipy.fft worker threads used by the transforms (the CPU baseline sets it).
WORKERS = 1

SUPP = 6  # delta support half-width in cells, src/streamfcn/structure-ops.jl:29


# ---------------------------------------------------------------------------
# Grid geometry: src/streamfcn/fluids.jl:23-45, src/fluids/fluids.jl:53-102
# ---------------------------------------------------------------------------
@dataclass
class Grid:
    """Sizes and BC offsets of ``StreamFcnGrid`` (src/streamfcn/fluids.jl:23-45)."""

    nx: int
    ny: int
    nlevels: int
    x0: float
    y0: float
    h: float

    def __post_init__(self):
        nx, ny = self.nx, self.ny
        if nx % 4 or ny % 4:
            raise ValueError("nx and ny must be divisible by 4 (fluid-ops.jl:189-232)")
        self.nu = (nx + 1) * ny
        self.nv = nx * (ny + 1)
        self.nq = self.nu + self.nv
        self.ngamma = (nx - 1) * (ny - 1)
        self.L = 0
        self.R = ny + 1
        self.B = 2 * (ny + 1)
        self.T = 2 * (ny + 1) + nx + 1
        self.nbc = 2 * (nx + 1) + 2 * (ny + 1)

    @property
    def gshape(self):
        return (self.ny - 1, self.nx - 1)

    def hc(self, lev: int) -> float:
        """``gridstep(grid, lev) = h * 2^(lev-1)`` (src/fluids/fluids.jl:102); lev is 1-based."""
        return self.h * 2.0 ** (lev - 1)


def grid_from_limits(h, xlims, ylims, nlevels):
    """``UniformGrid(h, (x0,x1), (y0,y1))`` (src/fluids/fluids.jl:53-56): ``x0:h:x1``."""
    def count(a, b):
        r = (b - a) / h
        n = round(r)
        if abs(r - n) > 1e-9 * max(1.0, abs(r)):
            n = math.floor(r)
        return int(n)
    return Grid(count(*xlims), count(*ylims), nlevels, float(xlims[0]), float(ylims[0]), float(h))


def split_flux(q, g: Grid):
    """``split_flux`` (src/streamfcn/fluids.jl:83-93): views of qx, qy in a flat q."""
    lead = q.shape[:-1]
    qx = q[..., : g.nu].reshape(*lead, g.ny, g.nx + 1)
    qy = q[..., g.nu:].reshape(*lead, g.ny + 1, g.nx)
    return qx, qy


def join_flux(qx, qy):
    lead = qx.shape[:-2]
    return np.concatenate([qx.reshape(*lead, -1), qy.reshape(*lead, -1)], axis=-1)


# ---------------------------------------------------------------------------
# Poisson solves: src/streamfcn/fluid-ops.jl:1-61
# ---------------------------------------------------------------------------
def dst2(x):
    """2-D DST-I, unnormalised (FFTW RODFT00 over both dims; fluid-ops.jl:25,49,51)."""
    return sfft.dstn(x, type=1, axes=(-2, -1), workers=WORKERS)


def lap_eigs(g: Grid):
    """``lap_eigs`` (fluid-ops.jl:58-61): -2(cos(pi i/nx) + cos(pi j/ny) - 2)."""
    i = np.arange(1, g.nx)
    j = np.arange(1, g.ny)
    ci = np.cos(np.pi * i / g.nx)
    cj = np.cos(np.pi * j / g.ny)
    return -2.0 * (ci[None, :] + cj[:, None] - 2.0)


def laplacian_inv(b, lam, g: Grid):
    """``LaplacianInv`` call (fluid-ops.jl:42-56): x = DST(DST(b) * scale/lam)."""
    scale = 1.0 / (4 * g.nx * g.ny)
    work = dst2(b)
    work = work * (scale / lam)
    return dst2(work)


def cn_multipliers(g: Grid, dt: float, Re: float):
    """``A_Ainv_linearmaps`` (src/streamfcn/cnab/ops.jl:14-42).

    Returns per level the eigen arrays handed to ``LaplacianInv``: A uses
    ``inv(1 - lam*dt/(2 Re hc^2))`` and Ainv uses ``1 + lam*dt/(2 Re hc^2)``
    (LaplacianInv divides by them).
    """
    lam = lap_eigs(g)
    expl, impl = [], []
    for lev in range(1, g.nlevels + 1):
        hc = g.hc(lev)
        expl.append(1.0 / (1.0 - lam * dt / (2 * Re * (hc * hc))))
        impl.append(1.0 + lam * dt / (2 * Re * (hc * hc)))
    return expl, impl


# ---------------------------------------------------------------------------
# Stencils: src/streamfcn/fluid-ops.jl:79-297
# ---------------------------------------------------------------------------
def curl0(psi, g: Grid):
    """Single-grid ``curl!`` with zero boundary (fluid-ops.jl:79-110)."""
    nx, ny = g.nx, g.ny
    lead = psi.shape[:-2]
    qx = np.zeros(lead + (ny, nx + 1))
    qy = np.zeros(lead + (ny + 1, nx))
    qx[..., 1:ny - 1, 1:nx] = psi[..., 1:ny - 1, 0:nx - 1] - psi[..., 0:ny - 2, 0:nx - 1]
    qx[..., 0, 1:nx] = psi[..., 0, 0:nx - 1]
    qx[..., ny - 1, 1:nx] = -psi[..., ny - 2, 0:nx - 1]
    qy[..., 1:ny, 1:nx - 1] = psi[..., 0:ny - 1, 0:nx - 2] - psi[..., 0:ny - 1, 1:nx - 1]
    qy[..., 1:ny, 0] = -psi[..., 0:ny - 1, 0]
    qy[..., 1:ny, nx - 1] = psi[..., 0:ny - 1, nx - 2]
    return join_flux(qx, qy)


def curl(psi, bc, g: Grid):
    """Multilevel ``curl!(q, psi, psibc)`` (fluid-ops.jl:138-182)."""
    nx, ny, L, R, B, T = g.nx, g.ny, g.L, g.R, g.B, g.T
    lead = psi.shape[:-2]
    qx = np.empty(lead + (ny, nx + 1))
    qy = np.empty(lead + (ny + 1, nx))
    qx[..., 1:ny - 1, 1:nx] = psi[..., 1:ny - 1, 0:nx - 1] - psi[..., 0:ny - 2, 0:nx - 1]
    qx[..., 0, 1:nx] = psi[..., 0, 0:nx - 1] - bc[..., B + 1:B + nx]
    qx[..., ny - 1, 1:nx] = bc[..., T + 1:T + nx] - psi[..., ny - 2, 0:nx - 1]
    qx[..., :, 0] = bc[..., L + 1:L + ny + 1] - bc[..., L:L + ny]
    qx[..., :, nx] = bc[..., R + 1:R + ny + 1] - bc[..., R:R + ny]
    qy[..., 1:ny, 1:nx - 1] = psi[..., 0:ny - 1, 0:nx - 2] - psi[..., 0:ny - 1, 1:nx - 1]
    qy[..., 1:ny, 0] = bc[..., L + 1:L + ny] - psi[..., 0:ny - 1, 0]
    qy[..., 1:ny, nx - 1] = psi[..., 0:ny - 1, nx - 2] - bc[..., R + 1:R + ny]
    qy[..., 0, :] = bc[..., B:B + nx] - bc[..., B + 1:B + nx + 1]
    qy[..., ny, :] = bc[..., T:T + nx] - bc[..., T + 1:T + nx + 1]
    return join_flux(qx, qy)


def rot(q, g: Grid):
    """``rot!`` = C^T (fluid-ops.jl:117-129)."""
    nx, ny = g.nx, g.ny
    qx, qy = split_flux(q, g)
    return (qx[..., 0:ny - 1, 1:nx] - qx[..., 1:ny, 1:nx]) + (
        qy[..., 1:ny, 1:nx] - qy[..., 1:ny, 0:nx - 1])


def coarsify(gc, gf, g: Grid):
    """``coarsify!`` (fluid-ops.jl:184-202): 9-point restriction into the coarse centre.

    Writes in place into ``gc`` and returns it.
    """
    nx, ny = g.nx, g.ny
    c = slice(1, ny - 2, 2), slice(1, nx - 2, 2)
    jp, jm = slice(2, ny - 1, 2), slice(0, ny - 3, 2)
    ip, im = slice(2, nx - 1, 2), slice(0, nx - 3, 2)
    f = gf
    val = (f[..., c[0], c[1]]
           + 0.5 * (f[..., c[0], ip] + f[..., jp, c[1]] + f[..., c[0], im] + f[..., jm, c[1]])
           + 0.25 * (f[..., jp, ip] + f[..., jm, ip] + f[..., jm, im] + f[..., jp, im]))
    gc[..., ny // 4:3 * ny // 4 - 1, nx // 4:3 * nx // 4 - 1] = val
    return gc


def get_bc(r, g: Grid):
    """``get_bc!`` (fluid-ops.jl:210-239): coarse-level values on the fine edge, times 0.25."""
    nx, ny, L, R, B, T = g.nx, g.ny, g.L, g.R, g.B, g.T
    nx4, ny4 = nx // 4, ny // 4
    lead = r.shape[:-2]
    bc = np.empty(lead + (g.nbc,))
    t = np.arange(nx // 2 + 1)
    bc[..., B + 2 * t] = r[..., ny4 - 1, nx4 - 1 + t]
    bc[..., T + 2 * t] = r[..., 3 * ny4 - 1, nx4 - 1 + t]
    t = np.arange(1, nx // 2 + 1)
    bc[..., B + 2 * t - 1] = 0.5 * (r[..., ny4 - 1, nx4 - 1 + t] + r[..., ny4 - 1, nx4 - 2 + t])
    bc[..., T + 2 * t - 1] = 0.5 * (r[..., 3 * ny4 - 1, nx4 - 1 + t]
                                    + r[..., 3 * ny4 - 1, nx4 - 2 + t])
    t = np.arange(ny // 2 + 1)
    bc[..., L + 2 * t] = r[..., ny4 - 1 + t, nx4 - 1]
    bc[..., R + 2 * t] = r[..., ny4 - 1 + t, 3 * nx4 - 1]
    t = np.arange(1, ny // 2 + 1)
    bc[..., L + 2 * t - 1] = 0.5 * (r[..., ny4 - 1 + t, nx4 - 1] + r[..., ny4 - 2 + t, nx4 - 1])
    bc[..., R + 2 * t - 1] = 0.5 * (r[..., ny4 - 1 + t, 3 * nx4 - 1]
                                    + r[..., ny4 - 2 + t, 3 * nx4 - 1])
    bc *= 0.25
    return bc


def apply_bc(r, bc, fac, g: Grid):
    """``apply_bc!`` (fluid-ops.jl:249-275): add ``fac * bc`` on the edge rows/columns, in place."""
    nx, ny, L, R, B, T = g.nx, g.ny, g.L, g.R, g.B, g.T
    r[..., 0, :] += fac * bc[..., B + 1:B + nx]
    r[..., ny - 2, :] += fac * bc[..., T + 1:T + nx]
    r[..., :, 0] += fac * bc[..., L + 1:L + ny]
    r[..., :, nx - 2] += fac * bc[..., R + 1:R + ny]
    return r


def avg_flux(q, q0, g: Grid):
    """``avg_flux!`` (fluid-ops.jl:277-297): face fluxes averaged to circulation nodes.

    Entries the reference leaves untouched (and never reads) are NaN here, so a
    stray read shows up in every downstream value.
    """
    nx, ny = g.nx, g.ny
    qx, qy = split_flux(q, g)
    q0x, q0y = split_flux(q0, g)
    Qx = np.full(qx.shape, np.nan)
    Qy = np.full(qy.shape, np.nan)
    Qx[..., 1:ny, :] = (qx[..., 1:ny, :] + qx[..., 0:ny - 1, :]
                        + q0x[..., 1:ny, :] + q0x[..., 0:ny - 1, :]) / 2
    Qy[..., :, 1:nx] = (qy[..., :, 1:nx] + qy[..., :, 0:nx - 1]
                        + q0y[..., :, 1:nx] + q0y[..., :, 0:nx - 1]) / 2
    return Qx, Qy


def direct_product(Qx, Qy, G, bc, g: Grid):
    """``direct_product!`` + loops (fluid-ops.jl:307-401): flux-circulation products."""
    nx, ny, L, R, B, T = g.nx, g.ny, g.L, g.R, g.B, g.T
    lead = G.shape[:-2]
    fqx = np.zeros(lead + (ny, nx + 1))
    fqy = np.zeros(lead + (ny + 1, nx))
    I = slice(1, nx)  # Julia i = 2:nx
    fqx[..., 1:ny - 1, I] = (Qy[..., 2:ny, I] * G[..., 1:ny - 1, 0:nx - 1]
                             + Qy[..., 1:ny - 1, I] * G[..., 0:ny - 2, 0:nx - 1]) / 2
    fqx[..., 0, I] = (Qy[..., 1, I] * G[..., 0, 0:nx - 1] + Qy[..., 0, I] * bc[..., B + 1:B + nx]) / 2
    fqx[..., ny - 1, I] = (Qy[..., ny - 1, I] * G[..., ny - 2, 0:nx - 1]
                           + Qy[..., ny, I] * bc[..., T + 1:T + nx]) / 2
    J = slice(1, ny)  # Julia j = 2:ny
    fqy[..., J, 1:nx - 1] = -(Qx[..., J, 2:nx] * G[..., 0:ny - 1, 1:nx - 1]
                              + Qx[..., J, 1:nx - 1] * G[..., 0:ny - 1, 0:nx - 2]) / 2
    fqy[..., J, 0] = -(Qx[..., J, 1] * G[..., 0:ny - 1, 0] + Qx[..., J, 0] * bc[..., L + 1:L + ny]) / 2
    fqy[..., J, nx - 1] = -(Qx[..., J, nx - 1] * G[..., 0:ny - 1, nx - 2]
                            + Qx[..., J, nx] * bc[..., R + 1:R + ny]) / 2
    return join_flux(fqx, fqy)


def nonlinear(q, q0, G, bc, lev, g: Grid):
    """``Nonlinear`` (cnab/ops.jl:151-167) via ``RhsForce`` (fluid-ops.jl:479-492)."""
    Qx, Qy = avg_flux(q, q0, g)
    fq = direct_product(Qx, Qy, G, bc, g)
    hc = g.hc(lev)
    return rot(fq, g) * (1 / (hc * hc))


def base_flux(g: Grid, u: float, v: float):
    """``base_flux!`` (fluid-ops.jl:403-417): q0 per level = (u hc, v hc)."""
    q0 = np.empty((g.nlevels, g.nq))
    for lev in range(1, g.nlevels + 1):
        hc = g.hc(lev)
        q0[lev - 1, : g.nu] = u * hc
        q0[lev - 1, g.nu:] = v * hc
    return q0


def vort2flux(G, g: Grid, lam):
    """``Vort2Flux`` (fluid-ops.jl:438-472).

    ``G`` has shape ``(..., nlevels, ny-1, nx-1)`` and is modified in place by the
    coarsening, like the reference.  Returns ``(psi, q)`` with ``q`` of shape
    ``(..., nlevels, nq)``.
    """
    nl = g.nlevels
    lead = G.shape[:-3]
    psi = np.zeros(G.shape)
    q = np.empty(lead + (nl, g.nq))
    for lev in range(2, nl + 1):
        coarsify(G[..., lev - 1, :, :], G[..., lev - 2, :, :], g)
    bc = np.zeros(lead + (g.nbc,))
    psi[..., nl - 1, :, :] = laplacian_inv(G[..., nl - 1, :, :], lam, g)
    q[..., nl - 1, :] = curl(psi[..., nl - 1, :, :], bc, g)
    for lev in range(nl - 1, 0, -1):
        tmp = G[..., lev - 1, :, :].copy()
        bc = get_bc(psi[..., lev, :, :], g)
        apply_bc(tmp, bc, 1.0, g)
        psi[..., lev - 1, :, :] = laplacian_inv(tmp, lam, g)
        q[..., lev - 1, :] = curl(psi[..., lev - 1, :, :], bc, g)
    return psi, q


# ---------------------------------------------------------------------------
# Regularized delta and E / E^T: src/streamfcn/structure-ops.jl:24-171
# ---------------------------------------------------------------------------
def delta_h(rf, rb, dr):
    """Yang-3 smooth delta ``δh`` times h (structure-ops.jl:114-171); same constants and order."""
    r = np.abs(np.asarray(rf, dtype=np.float64) - rb)
    r1 = r / dr
    r2 = r1 * r1
    r3 = r2 * r1
    r4 = r3 * r1
    out = np.zeros(np.broadcast(r1, r1).shape)
    s3 = math.sqrt(3.0)
    m1 = r1 <= 1.0
    m2 = (r1 > 1.0) & (r1 <= 2.0)
    m3 = (r1 > 2.0) & (r1 <= 3.0)
    if np.any(m1):
        a, b, c, d = r1[m1], r2[m1], r3[m1], r4[m1]
        a5 = np.arcsin((1.0 / 2.0) * s3 * (2.0 * a - 1.0))
        a8 = np.sqrt(1.0 - 12.0 * b + 12.0 * a)
        out[m1] = (4.166666667e-2 * d
                   + (-0.1388888889 + 3.472222222e-2 * a8) * c
                   + (-7.121664902e-2 - 5.208333333e-2 * a8 + 0.2405626122 * a5) * b
                   + (-0.2405626122 * a5 - 0.3792313933 + 0.1012731481 * a8) * a
                   + 8.0187537413e-2 * a5 - 4.195601852e-2 * a8 + 0.6485698427)
    if np.any(m2):
        a, b, c, d = r1[m2], r2[m2], r3[m2], r4[m2]
        a6 = np.arcsin((1.0 / 2.0) * s3 * (-3.0 + 2.0 * a))
        a9 = np.sqrt(-23.0 + 36.0 * a - 12.0 * b)
        out[m2] = (-6.250000000e-2 * d
                   + (0.4861111111 - 1.736111111e-2 * a9) * c
                   + (-1.143175026 + 7.812500000e-2 * a9 - 0.1202813061 * a6) * b
                   + (0.8751991178 + 0.3608439183 * a6 - 0.1548032407 * a9) * a
                   - 0.2806563809 * a6 + 8.22848104e-3 + 0.1150173611 * a9)
    if np.any(m3):
        a, b, c, d = r1[m3], r2[m3], r3[m3], r4[m3]
        a1 = np.arcsin((1.0 / 2.0 * (2.0 * a - 5.0)) * s3)
        a7 = np.sqrt(-71.0 - 12.0 * b + 60.0 * a)
        out[m3] = (2.083333333e-2 * d
                   + (3.472222222e-3 * a7 - 0.2638888889) * c
                   + (1.214391675 - 2.604166667e-2 * a7 + 2.405626122e-2 * a1) * b
                   + (-0.1202813061 * a1 - 2.449273192 + 7.262731481e-2 * a7) * a
                   + 0.1523563211 * a1 + 1.843201677 - 7.306134259e-2 * a7)
    return out


@dataclass
class Reg:
    """``Reg`` (structure-ops.jl:4-9): per-point 13x13 weights for the qx and qy grids.

    ``body_idx``: (nb, 2) of ``floor((xb - x0)/h)`` (Julia face index of the window centre).
    ``weight``: (nb, 2, 13, 13) indexed ``[k, component, b (y offset), a (x offset)]``.
    """

    body_idx: np.ndarray
    weight: np.ndarray


def reg_update(xb, g: Grid) -> Reg:
    """``Reg`` + ``update!`` (structure-ops.jl:24-61)."""
    xb = np.asarray(xb, dtype=np.float64)
    h = g.h
    x0, y0 = g.x0, g.y0
    bi = np.floor((xb[:, 0] - x0) / h).astype(np.int64)
    bj = np.floor((xb[:, 1] - y0) / h).astype(np.int64)
    s = np.arange(-SUPP, SUPP + 1)
    x = h * (bi[:, None] - 1 + s[None, :]) + x0        # (nb, 13) over a
    y = h * (bj[:, None] - 1 + s[None, :]) + y0        # (nb, 13) over b
    xk = xb[:, 0][:, None]
    yk = xb[:, 1][:, None]
    w = np.empty((xb.shape[0], 2, 2 * SUPP + 1, 2 * SUPP + 1))
    w[:, 0] = delta_h(y + h / 2, yk, h)[:, :, None] * delta_h(x, xk, h)[:, None, :]
    w[:, 1] = delta_h(y, yk, h)[:, :, None] * delta_h(x + h / 2, xk, h)[:, None, :]
    return Reg(np.stack([bi, bj], axis=1), w)


def _windows(reg: Reg, g: Grid):
    """0-based (j, i) window origins for point k: Julia face index ``body_idx + s``, s=-6..6."""
    nb = reg.body_idx.shape[0]
    i0 = reg.body_idx[:, 0] - SUPP - 1
    j0 = reg.body_idx[:, 1] - SUPP - 1
    n = 2 * SUPP + 1
    if nb and (i0.min() < 0 or j0.min() < 0 or i0.max() + n > g.nx or j0.max() + n > g.ny):
        raise IndexError("body point within 7 cells of the finest-grid edge")
    return i0, j0


def reg_scatter(fb, reg: Reg, g: Grid):
    """E^T: ``(reg::Reg)(q, fb)`` (structure-ops.jl:63-86); k-ordered accumulation."""
    nb = reg.body_idx.shape[0]
    fb = np.asarray(fb)
    lead = fb.shape[:-1]
    q = np.zeros(lead + (g.nq,))
    qx, qy = split_flux(q, g)
    i0, j0 = _windows(reg, g)
    n = 2 * SUPP + 1
    for k in range(nb):
        sj, si = slice(j0[k], j0[k] + n), slice(i0[k], i0[k] + n)
        qx[..., sj, si] += reg.weight[k, 0] * fb[..., k, None, None]
        qy[..., sj, si] += reg.weight[k, 1] * fb[..., nb + k, None, None]
        if not np.all(np.isfinite(np.sum(qx[..., sj, si] ** 2, axis=(-2, -1)))):
            raise FloatingPointError("infinite flux")
    return q


def reg_gather(q, reg: Reg, g: Grid):
    """E: ``(regT::RegT)(fb, q)`` (structure-ops.jl:88-105)."""
    nb = reg.body_idx.shape[0]
    qx, qy = split_flux(q, g)
    i0, j0 = _windows(reg, g)
    n = 2 * SUPP + 1
    lead = q.shape[:-1]
    fb = np.zeros(lead + (2 * nb,))
    ar = np.arange(n)
    jj = j0[:, None, None] + ar[None, :, None]
    ii = i0[:, None, None] + ar[None, None, :]
    wx = qx[..., jj, ii]  # (..., nb, 13, 13)
    wy = qy[..., jj, ii]
    fb[..., :nb] = np.sum(wx * reg.weight[:, 0], axis=(-2, -1))
    fb[..., nb:] = np.sum(wy * reg.weight[:, 1], axis=(-2, -1))
    return fb


# ---------------------------------------------------------------------------
# Schur complement: src/streamfcn/cnab/ops.jl:44-143
# ---------------------------------------------------------------------------
def b_times(z, reg: Reg, g: Grid, lam, ainv1):
    """``B_Times`` (cnab/ops.jl:125-143): x = E q1(vort2flux(Ainv1 C^T E^T z)); z may be batched."""
    z = np.asarray(z, dtype=np.float64)
    lead = z.shape[:-1]
    G = np.zeros(lead + (g.nlevels,) + g.gshape)
    qtmp = reg_scatter(z, reg, g)
    gtmp = rot(qtmp, g)
    G[..., 0, :, :] = laplacian_inv(gtmp, ainv1, g)
    _, q = vort2flux(G, g, lam)
    return reg_gather(q[..., 0, :], reg, g)


def schur_matrix(reg: Reg, g: Grid, lam, ainv1, batch: int = 64):
    """``Bmat[:, j] = B e_j`` (cnab/ops.jl:79-94), assembled ``batch`` columns at a time."""
    nf = 2 * reg.body_idx.shape[0]
    Bmat = np.empty((nf, nf))
    for c0 in range(0, nf, batch):
        c1 = min(nf, c0 + batch)
        E = np.zeros((c1 - c0, nf))
        E[np.arange(c1 - c0), np.arange(c0, c1)] = 1.0
        Bmat[:, c0:c1] = b_times(E, reg, g, lam, ainv1).T
    return Bmat


# ---------------------------------------------------------------------------
# Problem, state, CNAB step: src/streamfcn/cnab/timestepping.jl, states.jl
# ---------------------------------------------------------------------------
@dataclass
class Problem:
    """Plain-parameter form of ``Problem(StreamFcnFluid(...), BodyGroup(...), SchemeCNAB(dt))``."""

    grid: Grid
    dt: float
    Re: float
    xb: np.ndarray                      # (nb, 2) stacked body points
    ds: np.ndarray                      # (nb,) segment lengths
    body_npoints: list                  # points per body
    beta: tuple = (1.5, -0.5)           # SchemeCNAB(Val(2), dt), src/schemes.jl:22
    freestream: object = (1.0, 0.0)     # (u, v) constant or callable t -> (u, v)
    grid_velocity: object = None        # translating grid: t -> (vx, vy) of the grid frame

    def uv(self, t):
        """The uniform flow of base_flux! (fluid-ops.jl:403-417) in grid coordinates: the
        freestream, minus the grid's velocity when the grid translates (the moving-grid case the
        reference leaves as a TODO at fluid-ops.jl:419, restated as a Galilean change of frame)."""
        f = self.freestream
        u, v = tuple(f(t)) if callable(f) else tuple(f)
        if self.grid_velocity is not None:
            gx, gy = self.grid_velocity(t)
            u, v = u - gx, v - gy
        return (u, v)


@dataclass
class State:
    """``CNAB.State`` (cnab/states.jl:1-16) with ``StreamFcnQuantities`` (states.jl:9-41)."""

    gamma: np.ndarray      # (L, ny-1, nx-1)
    psi: np.ndarray        # (L, ny-1, nx-1)
    q: np.ndarray          # (L, nq)
    q0: np.ndarray         # (L, nq)
    fb: np.ndarray         # (2 nb,)
    nonlin: list           # [newest, previous], each (L, ny-1, nx-1)
    t: float
    cd: np.ndarray = field(default_factory=lambda: np.zeros(0))
    cl: np.ndarray = field(default_factory=lambda: np.zeros(0))
    stress: list = field(default_factory=list)

    def copy(self):
        return State(self.gamma.copy(), self.psi.copy(), self.q.copy(), self.q0.copy(),
                     self.fb.copy(), [a.copy() for a in self.nonlin], self.t,
                     self.cd.copy(), self.cl.copy(), [s.copy() for s in self.stress])


def init_state(prob: Problem, t: float = 0.0) -> State:
    """``initstate`` -> ``State(prob, t)`` (cnab/states.jl:8-16, states.jl:19-41)."""
    g = prob.grid
    L = g.nlevels
    shp = (L,) + g.gshape
    nbod = len(prob.body_npoints)
    st = State(np.zeros(shp), np.zeros(shp), np.zeros((L, g.nq)),
               base_flux(g, *prob.uv(t)), np.zeros(2 * int(sum(prob.body_npoints))),
               [np.zeros(shp), np.zeros(shp)], float(t), np.zeros(nbod), np.zeros(nbod),
               [np.zeros((n, 2)) for n in prob.body_npoints])
    return st


class Solver:
    """``CNAB.Solver`` (cnab/timestepping.jl:193-249): setup of all operators for static bodies."""

    def __init__(self, prob: Problem, state: State | None = None, assemble: bool = True,
                 batch: int = 64, precond=None):
        """``assemble``: build ``Bmat`` column by column and invert it (the reference's setup,
        ``batch`` columns per bulk solve).  ``precond``: instead of the dense inverse, solve
        B Fb = E Q every step by preconditioned iterative refinement on this oracle's own
        matrix-free ``B_Times`` (``schur_solve``); the matrix given only speeds convergence, the
        answer is this oracle's B^-1 E Q to the refinement's tolerance.  Used where assembling
        nf columns of full-size transforms on the CPU takes too long for a test."""
        g = prob.grid
        self.prob = prob
        self.g = g
        self.lam = lap_eigs(g)
        self.expl, self.impl = cn_multipliers(g, prob.dt, prob.Re)
        self.reg = reg_update(prob.xb, g)
        self.P = None
        self.refine_iterations = []
        if precond is not None:
            self.Bmat = None
            self.Binv = None
            self.P = np.asarray(precond, dtype=np.float64)
        elif assemble:
            self.Bmat = schur_matrix(self.reg, g, self.lam, self.impl[0], batch=batch)
            self.Binv = np.linalg.inv(self.Bmat)
        else:
            # timing only: a stand-in inverse of the right shape (the per-step work of the
            # dense matvec is the same; forces are not meaningful)
            nf = 2 * self.reg.body_idx.shape[0]
            self.Bmat = None
            self.Binv = np.random.default_rng(0).standard_normal((nf, nf)) * 1e-6

    # --- GetTrialState (cnab/timestepping.jl:28-79) ---------------------------------
    def trial_state(self, st: State):
        g, prob = self.g, self.prob
        L = g.nlevels
        dt, Re = prob.dt, prob.Re
        gs = np.empty_like(st.gamma)
        bc = np.zeros(g.nbc)
        rhsbc = np.zeros(g.gshape)
        new_nl = np.empty_like(st.gamma)
        for lev in range(L, 0, -1):
            hc = g.hc(lev)
            if lev < L:
                bc = get_bc(st.gamma[lev], g)
                fac = 0.25 * dt / (Re * (hc * hc))
                apply_bc(rhsbc, bc, fac, g)
            bc = bc * 0.25
            new_nl[lev - 1] = nonlinear(st.q[lev - 1], st.q0[lev - 1], st.gamma[lev - 1], bc, lev, g)
            rhs = laplacian_inv(st.gamma[lev - 1], self.expl[lev - 1], g)
            rhs = rhs + dt * prob.beta[0] * new_nl[lev - 1]
            rhs = rhs + dt * prob.beta[1] * st.nonlin[1][lev - 1]
            rhs = rhs + rhsbc
            gs[lev - 1] = laplacian_inv(rhs, self.impl[lev - 1], g)
        # nonlin[1] holds the new term during the level loop; cycle! makes it the
        # history: after the step nonlin = [old history slot, new term].
        st.nonlin = [st.nonlin[1], new_nl]
        psi, qs = vort2flux(gs, g, self.lam)
        st.psi = psi
        return qs, gs

    def advance(self, st: State, t: float):
        """``advance!`` (cnab/timestepping.jl:253-290) for bodies fixed in the grid frame."""
        g, prob = self.g, self.prob
        st.q0 = base_flux(g, *prob.uv(t))
        qs, gs = self.trial_state(st)
        # BoundaryForcer{RigidBody{GridFrame}} (timestepping.jl:106-120)
        Q = qs[0] + st.q0[0]
        ftmp = reg_gather(Q, self.reg, g)
        if self.P is not None:
            apply_B = lambda z: b_times(z, self.reg, g, self.lam, self.impl[0])
            st.fb, it, _ = schur_solve(apply_B, self.P, ftmp, self.P @ ftmp)
            self.refine_iterations.append(it)
        else:
            st.fb = self.Binv @ ftmp
        update_stress(st, prob)
        # CircProjecter (timestepping.jl:156-171)
        st.gamma = gs.copy()
        qtmp = reg_scatter(st.fb, self.reg, g)
        gtmp = rot(qtmp, g)
        st.gamma[0] -= laplacian_inv(gtmp, self.impl[0], g)
        # Vort2Flux on the state (timestepping.jl:285)
        st.psi, st.q = vort2flux(st.gamma, g, self.lam)
        st.t = float(t)


def update_stress(st: State, prob: Problem):
    """``update_stress!`` (src/streamfcn/states.jl:53-84)."""
    g = prob.grid
    nb = int(sum(prob.body_npoints))
    F = st.fb.reshape(2, nb).T
    h, dt = g.h, prob.dt
    cd, cl, stress = [], [], []
    i = 0
    for n in prob.body_npoints:
        fb = F[i:i + n] * h / dt
        cd.append(2 * np.sum(fb[:, 0]))
        cl.append(2 * np.sum(fb[:, 1]))
        stress.append(fb / prob.ds[i:i + n, None])
        i += n
    st.cd, st.cl, st.stress = np.array(cd), np.array(cl), stress


def solve(prob: Problem, st: State, t0: float, nsteps: int, solver: Solver | None = None,
          record=None):
    """``solve!`` time loop (src/solve.jl:188-215): ``advance!`` at t0, t0+dt, ... (t0 included).

    ``record(i, state)`` is called after every step (1-based i).
    """
    solver = solver or Solver(prob, st)
    for i in range(nsteps):
        t = t0 + i * prob.dt
        solver.advance(st, t)
        if record is not None:
            record(i + 1, st)
    return solver


# ---------------------------------------------------------------------------
# Moving bodies (corrected restatement): src/bodies/body-points.jl:47-76,
# src/streamfcn/cnab/timestepping.jl:122-139, src/streamfcn/cnab/ops.jl:104-114.
#
# The reference's moving-body branch cannot run (update_bodies! reads a field :ω that
# RelativeFrame names Ω, copies positions into velocities, and a LabFrame fluid keeps a
# stale dense Binv).  This restatement applies the evident fixes:
#   * r = r0 + R(θ) xb,  v = v0 + Ω R'(θ) xb      (body-points.jl:49-65, field Ω)
#   * the stacked velocities are the points' v    (body-points.jl:73)
#   * E / E^T weights rebuilt every step           (structure-ops.jl:37-61)
#   * Fb solves B Fb = E(qs + q0) - ub h by CG      (timestepping.jl:122-139, ops.jl:104-114),
#     warm-started from the previous Fb like cg!(qty.Fb, ...), stopping when
#     ||r|| <= tol ||rhs|| (tol 1e-10; the reference's reltol is relative to the first residual)
# ---------------------------------------------------------------------------
def rigid_motion(xb_body, r0, v0, theta, omega):
    """Positions and velocities of body-frame points xb_body (n, 2) under a rigid motion."""
    c, s = math.cos(theta), math.sin(theta)
    R = np.array([[c, -s], [s, c]])
    Rv = omega * np.array([[-s, -c], [c, -s]])
    r = np.asarray(r0)[None, :] + xb_body @ R.T
    v = np.asarray(v0)[None, :] + xb_body @ Rv.T
    return r, v


def cg_solve(apply_B, rhs, x0, tol=1e-10, maxiter=5000):
    """Unpreconditioned conjugate gradients (the iteration of IterativeSolvers.cg!, 0.9.2).

    Stops when ||b - A x|| <= tol * ||b||.  Returns (x, iterations, residual norm)."""
    x = np.array(x0, dtype=np.float64)
    r = rhs - apply_B(x)
    bn = np.linalg.norm(rhs)
    target = tol * bn
    rr = float(r @ r)
    if math.sqrt(rr) <= target:
        return x, 0, math.sqrt(rr)
    p = r.copy()
    for it in range(1, maxiter + 1):
        Ap = apply_B(p)
        alpha = rr / float(p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        rr_new = float(r @ r)
        if math.sqrt(rr_new) <= target:
            return x, it, math.sqrt(rr_new)
        p = r + (rr_new / rr) * p
        rr = rr_new
    return x, maxiter, math.sqrt(rr)


def schur_solve(apply_B, P, rhs, x0, tol=1e-14, maxiter=60):
    """Solve B x = rhs by iterative refinement preconditioned with P ~ B^-1:
    x += P (rhs - B x) until ||rhs - B x|| <= tol ||rhs|| or the residual stops falling
    (its floor is the rounding of B x).  The answer is determined by ``apply_B`` alone; P only
    sets the rate.  Returns (x, iterations, relative residual)."""
    x = np.array(x0, dtype=np.float64)
    bn = np.linalg.norm(rhs)
    r = rhs - apply_B(x)
    rn = np.linalg.norm(r)
    best = (rn, x.copy())
    it = 0
    stalled = 0
    while rn > tol * bn and it < maxiter:
        x = x + P @ r
        r = rhs - apply_B(x)
        rn = np.linalg.norm(r)
        it += 1
        if rn < 0.5 * best[0]:
            best, stalled = (rn, x.copy()), 0
        else:
            stalled += 1
            if rn < best[0]:
                best = (rn, x.copy())
            if stalled >= 3:
                break
    return best[1], it, best[0] / (bn if bn > 0 else 1.0)


@dataclass
class MovingProblem:
    """A problem whose bodies move rigidly: ``kinematics(t) -> [(r0, v0, θ, Ω) per body]``."""

    grid: Grid
    dt: float
    Re: float
    xb_body: list            # per body (n_b, 2) body-frame points
    ds: np.ndarray           # (nb,) stacked segment lengths
    kinematics: object
    beta: tuple = (1.5, -0.5)
    freestream: object = (1.0, 0.0)
    cg_tol: float = 1e-10
    cg_maxiter: int = 5000

    @property
    def body_npoints(self):
        return [x.shape[0] for x in self.xb_body]

    def uv(self, t):
        f = self.freestream
        return tuple(f(t)) if callable(f) else tuple(f)

    def points(self, t):
        rs, vs = [], []
        for xb, (r0, v0, th, om) in zip(self.xb_body, self.kinematics(t)):
            r, v = rigid_motion(xb, r0, v0, th, om)
            rs.append(r)
            vs.append(v)
        return np.concatenate(rs), np.concatenate(vs)


class MovingSolver(Solver):
    """``advance!`` for moving bodies with the corrections listed above."""

    def __init__(self, prob: MovingProblem, precondition: bool = False, batch: int = 64):
        """``precondition``: solve each step's B Fb = rhs by iterative refinement with the
        inverse of this oracle's own Schur matrix assembled at the first step's body positions
        (``schur_solve``) instead of plain CG; the answer is the same system's solution, reached
        in a few B products instead of the ~10^3 CG iterations that cond(B) ~ 1e5 needs."""
        g = prob.grid
        self.prob = prob
        self.g = g
        self.lam = lap_eigs(g)
        self.expl, self.impl = cn_multipliers(g, prob.dt, prob.Re)
        self.cg_iterations = []
        self.precondition = precondition
        self.batch = batch
        self.P = None

    def advance(self, st: State, t: float, warm=None):
        g, prob = self.g, self.prob
        xb, vb = prob.points(t)                       # update_bodies!
        self.reg = reg_update(xb, g)                  # update!(reg, points)
        st.q0 = base_flux(g, *prob.uv(t))
        qs, gs = self.trial_state(st)
        Q = qs[0] + st.q0[0]
        ftmp = reg_gather(Q, self.reg, g) - np.concatenate([vb[:, 0], vb[:, 1]]) * g.h
        x0 = st.fb if warm is None else warm
        apply_B = lambda z: b_times(z, self.reg, g, self.lam, self.impl[0])
        if self.precondition:
            if self.P is None:
                self.P = np.linalg.inv(schur_matrix(self.reg, g, self.lam, self.impl[0], batch=self.batch))
            st.fb, it, res = schur_solve(apply_B, self.P, ftmp, x0, tol=prob.cg_tol)
        else:
            st.fb, it, res = cg_solve(apply_B, ftmp, x0, prob.cg_tol, prob.cg_maxiter)
        self.cg_iterations.append(it)
        update_stress(st, prob)
        st.gamma = gs.copy()
        qtmp = reg_scatter(st.fb, self.reg, g)
        st.gamma[0] -= laplacian_inv(rot(qtmp, g), self.impl[0], g)
        st.psi, st.q = vort2flux(st.gamma, g, self.lam)
        st.t = float(t)
        st.points, st.velocities = xb, vb


# ---------------------------------------------------------------------------
# Checkpoint files of libibgb300 (ib_checkpoint_save / ib_checkpoint_load): the reference keeps
# snapshots in memory only (copy! of the state, states.jl:90-112, cnab/states.jl:23-27); this
# reader lets the oracle continue a run the GPU saved, and the writer makes files for tests.
# Layout: 56-byte header (8-byte magic "IBGB300C", int32 version 1, nx, ny, nlevels, npoints,
# moving flag, two int32 zeros, float64 t, int64 steps) then float64 arrays in the column-major
# layouts: Gamma, q, psi, nonlin[1], nonlin[2], Fb [, previous Fb when moving].
# ---------------------------------------------------------------------------
_CKPT_HEADER = np.dtype([("magic", "S8"), ("version", "<i4"), ("nx", "<i4"), ("ny", "<i4"), ("nlevels", "<i4"),
                         ("npoints", "<i4"), ("moving", "<i4"), ("r0", "<i4"), ("r1", "<i4"), ("t", "<f8"),
                         ("steps", "<i8")])


def write_checkpoint(path, g: Grid, st: State, steps: int = 0, fb_prev=None):
    """Write an oracle State in the libibgb300 checkpoint layout."""
    L = g.nlevels
    hd = np.zeros(1, dtype=_CKPT_HEADER)
    nb = st.fb.size // 2
    hd[0] = (b"IBGB300C", 1, g.nx, g.ny, L, nb, 1 if fb_prev is not None else 0, 0, 0, st.t, steps)
    parts = [st.gamma.reshape(L, -1), st.q.reshape(L, -1), st.psi.reshape(L, -1),
             st.nonlin[0].reshape(L, -1), st.nonlin[1].reshape(L, -1), st.fb]
    if fb_prev is not None:
        parts.append(np.asarray(fb_prev))
    with open(path, "wb") as f:
        f.write(hd.tobytes())
        for a in parts:
            f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())


def read_checkpoint(path, g: Grid) -> dict:
    """Read a libibgb300 checkpoint for grid g: header fields and the arrays, shaped like the
    oracle's State fields (``nonlin`` as [older, newest] like ``State.nonlin``: the file's
    nonlin[1] and nonlin[2] in the reference's 1-based order)."""
    raw = open(path, "rb").read()
    hd = np.frombuffer(raw[:_CKPT_HEADER.itemsize], dtype=_CKPT_HEADER)[0]
    if hd["magic"] != b"IBGB300C" or hd["version"] != 1:
        raise ValueError("not a version-1 libibgb300 checkpoint")
    if (hd["nx"], hd["ny"], hd["nlevels"]) != (g.nx, g.ny, g.nlevels):
        raise ValueError("checkpoint grid differs from the problem's")
    L, nb = g.nlevels, int(hd["npoints"])
    v = np.frombuffer(raw[_CKPT_HEADER.itemsize:], dtype="<f8")
    sizes = [L * g.ngamma, L * g.nq, L * g.ngamma, L * g.ngamma, L * g.ngamma, 2 * nb]
    if hd["moving"]:
        sizes.append(2 * nb)
    if v.size != sum(sizes):
        raise ValueError("checkpoint size differs from its header")
    out, o = [], 0
    for n in sizes:
        out.append(v[o:o + n].copy())
        o += n
    shp = (L,) + g.gshape
    return {"t": float(hd["t"]), "steps": int(hd["steps"]), "gamma": out[0].reshape(shp),
            "q": out[1].reshape(L, g.nq), "psi": out[2].reshape(shp),
            "nonlin": [out[3].reshape(shp), out[4].reshape(shp)], "fb": out[5],
            "fb_prev": out[6] if hd["moving"] else None}


def state_from_checkpoint(prob: Problem, ck: dict) -> State:
    """An oracle State continuing from a checkpoint (q0 is recomputed by the next advance)."""
    st = init_state(prob, ck["t"])
    st.gamma, st.q, st.psi = ck["gamma"].copy(), ck["q"].copy(), ck["psi"].copy()
    st.nonlin = [a.copy() for a in ck["nonlin"]]
    st.fb = ck["fb"].copy()
    return st


# ---------------------------------------------------------------------------
# SchemeRKC (src/schemes.jl:3-12, "Runge-Kutta-Chebyshev scheme"): declared by the reference,
# which defines no state or solver for it.  This is the definition libibgb300 implements
# (IB_SCHEME_RKC), restated: the s-stage second-order RKC method with damping eps = 2/13
# (Sommeijer, Shampine & Verwer 1998) on dGamma/dt = F(Gamma), per level
#   F_l = N_l(Gamma) + (1 / (Re hc_l^2)) (apply_bc(get_bc(Gamma_{l+1})) - lap5(Gamma_l)),
# N_l the CNAB scheme's nonlinear term with its rings (cnab/ops.jl:151-167, timestepping.jl:
# 48-58), then the projection Gamma_1 -= C^T E^T Fb with Fb = B'^-1 E(q1 + q0),
# B' = E C Lap^-1 C^T E^T (B_Times without the implicit operator).
# ---------------------------------------------------------------------------
def rkc_coefficients(S: int):
    """(mu, nu, mut, gamt, beta): stage coefficients indexed 1..S and the stability interval."""
    eps = 2.0 / 13.0
    w0 = 1.0 + eps / (S * S)
    T, T1, T2 = [1.0, w0], [0.0, 1.0], [0.0, 0.0]
    for j in range(2, S + 1):
        T.append(2 * w0 * T[j - 1] - T[j - 2])
        T1.append(2 * T[j - 1] + 2 * w0 * T1[j - 1] - T1[j - 2])
        T2.append(4 * T1[j - 1] + 2 * w0 * T2[j - 1] - T2[j - 2])
    w1 = T1[S] / T2[S]
    b = [0.0] * (S + 1)
    for j in range(2, S + 1):
        b[j] = T2[j] / T1[j] ** 2
    b[0] = b[1] = b[2]
    mu, nu, mut, gamt = [0.0] * (S + 1), [0.0] * (S + 1), [0.0] * (S + 1), [0.0] * (S + 1)
    mut[1] = b[1] * w1
    for j in range(2, S + 1):
        mu[j] = 2 * b[j] * w0 / b[j - 1]
        nu[j] = -b[j] / b[j - 2]
        mut[j] = 2 * b[j] * w1 / b[j - 1]
        gamt[j] = -(1 - b[j - 1] * T[j - 1]) * mut[j]
    return mu, nu, mut, gamt, (w0 + 1) * T2[S] / T1[S]


def lap5(Y):
    """4 Y - (its four neighbours), zero outside the array (rot o curl with zero ring)."""
    out = 4.0 * Y
    out[..., :, 1:] -= Y[..., :, :-1]
    out[..., :, :-1] -= Y[..., :, 1:]
    out[..., 1:, :] -= Y[..., :-1, :]
    out[..., :-1, :] -= Y[..., 1:, :]
    return out


def b_times_explicit(z, reg: Reg, g: Grid, lam):
    """B' z = E q1(vort2flux(C^T E^T z)) (B_Times, cnab/ops.jl:125-143, without Ainv)."""
    z = np.asarray(z, dtype=np.float64)
    lead = z.shape[:-1]
    G = np.zeros(lead + (g.nlevels,) + g.gshape)
    G[..., 0, :, :] = rot(reg_scatter(z, reg, g), g)
    _, q = vort2flux(G, g, lam)
    return reg_gather(q[..., 0, :], reg, g)


class RKCSolver(Solver):
    """SchemeRKC restated (see above): bodies fixed in the grid, FP64."""

    def __init__(self, prob: Problem, stages: int = 0, batch: int = 64):
        g = prob.grid
        self.prob, self.g = prob, g
        self.lam = lap_eigs(g)
        self.reg = reg_update(prob.xb, g)
        nf = 2 * self.reg.body_idx.shape[0]
        if nf:
            B = np.empty((nf, nf))
            for c0 in range(0, nf, batch):
                c1 = min(nf, c0 + batch)
                E = np.zeros((c1 - c0, nf))
                E[np.arange(c1 - c0), np.arange(c0, c1)] = 1.0
                B[:, c0:c1] = b_times_explicit(E, self.reg, g, self.lam).T
            self.Bmat, self.Binv = B, np.linalg.inv(B)
        else:
            self.Bmat = self.Binv = np.zeros((0, 0))
        if stages == 0:
            need = 1.5 * prob.dt * 8.0 / (prob.Re * g.h * g.h)
            stages = 2
            while stages < 64 and rkc_coefficients(stages)[4] < need:
                stages += 1
        self.stages = stages
        self.coef = rkc_coefficients(stages)

    def F(self, Y, q, q0):
        g, prob = self.g, self.prob
        L = g.nlevels
        out = np.empty_like(Y)
        for lev in range(1, L + 1):
            bcv = get_bc(Y[lev], g) if lev < L else np.zeros(g.nbc)
            nl = nonlinear(q[lev - 1], q0[lev - 1], Y[lev - 1], 0.25 * bcv, lev, g)
            visc = -lap5(Y[lev - 1])
            apply_bc(visc, bcv, 1.0, g)
            hc = g.hc(lev)
            out[lev - 1] = nl + visc / (prob.Re * hc * hc)
        return out

    def advance(self, st: State, t: float):
        g, prob = self.g, self.prob
        dt = prob.dt
        mu, nu, mut, gamt, _ = self.coef
        st.q0 = base_flux(g, *prob.uv(t))
        Y0 = st.gamma.copy()
        F0 = self.F(Y0, st.q, st.q0)
        Ym2, Ym1 = Y0, Y0 + mut[1] * dt * F0
        for j in range(2, self.stages + 1):
            _, q = vort2flux(Ym1, g, self.lam)
            Fj = self.F(Ym1, q, st.q0)
            Yj = (1 - mu[j] - nu[j]) * Y0 + mu[j] * Ym1 + nu[j] * Ym2 + mut[j] * dt * Fj + gamt[j] * dt * F0
            Ym2, Ym1 = Ym1, Yj
        out = Ym1
        if self.Binv.size:
            _, qs = vort2flux(out, g, self.lam)
            ftmp = reg_gather(qs[0] + st.q0[0], self.reg, g)
            st.fb = self.Binv @ ftmp
            update_stress(st, prob)
            out[0] -= rot(reg_scatter(st.fb, self.reg, g), g)
        st.gamma = out
        st.psi, st.q = vort2flux(st.gamma, g, self.lam)
        st.t = float(t)
