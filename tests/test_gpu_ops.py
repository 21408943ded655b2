"""Operator-level parity: each libibgb300 operator entry point (include/ibgb300_ops.h) against
the FP64 oracle on the same seeded inputs."""
import numpy as np
import pytest
from scipy import fft as sfft

from _util import Dev, rel

pytestmark = pytest.mark.gpu

TOL = 1e-12  # FP64 operators: relative L2 (transforms: a few ulps times log n)


@pytest.fixture(scope="module")
def dev():
    pytest.importorskip("torch")
    return Dev()


def make(ib, nx, ny, L, bodies=()):
    h = 4.0 / nx
    grid = ib.MultiLevel(ib.UniformGrid(h, (-1.0, -1.0 + nx * h), (-0.5 * ny * h, 0.5 * ny * h)), L)
    prob = ib.Problem(ib.StreamFcnFluid(grid, (1.0, 0.0), 100.0), ib.BodyGroup(*bodies), ib.SchemeCNAB(0.01))
    st = ib.initstate(prob)
    return prob, ib.initsolver(prob, st)


def ogrid(O, prob):
    d = prob.fluid.domain
    b = d.discrete.base
    return O.Grid(b.nx, b.ny, d.discrete.nlevels, float(b.xs[0]), float(b.ys[0]), b.h)


# IBGB300_DST=warp: axes of 64 P cells (P = 2^k or 3 2^k, P <= 32) on both sides run the
# warp-per-line passes, the others the shared-memory Stockham passes
@pytest.mark.parametrize("dst", ["warp", "stockham"])
@pytest.mark.parametrize("nx,ny", [(16, 24), (40, 32), (200, 200), (256, 384), (1024, 768), (2048, 64),
                                   (256, 128), (64, 2048), (1024, 1024), (768, 512), (192, 1536)])
def test_dst2_matches_rodft00(ib, lib, dev, monkeypatch, nx, ny, dst):
    monkeypatch.setenv("IBGB300_DST", dst)
    prob, s = make(ib, nx, ny, 1)
    rng = np.random.default_rng(nx + ny)
    x = rng.standard_normal((3, ny - 1, nx - 1))
    dx, dy = dev.put(x), dev.empty(x.size)
    assert lib.ib_op_dst2(s.handle, 3, dev.p(dx), dev.p(dy)) == 0
    got = dev.get(dy).reshape(x.shape)
    want = sfft.dstn(x, type=1, axes=(-2, -1))
    assert np.max(np.abs(got - want)) / np.max(np.abs(want)) < 1e-13
    s.close()


def test_dst2_pure_mode(ib, lib, dev):
    nx, ny = 64, 48
    prob, s = make(ib, nx, ny, 1)
    I = np.arange(1, nx)[None, :]
    J = np.arange(1, ny)[:, None]
    x = np.sin(np.pi * 5 * I / nx) * np.sin(np.pi * 7 * J / ny)
    dx, dy = dev.put(x), dev.empty(x.size)
    assert lib.ib_op_dst2(s.handle, 1, dev.p(dx), dev.p(dy)) == 0
    got = dev.get(dy).reshape(x.shape)
    want = np.zeros_like(x)
    want[6, 4] = nx * ny
    assert np.max(np.abs(got - want)) < 1e-10 * nx * ny
    s.close()


@pytest.mark.parametrize("dst", ["warp", "stockham"])
@pytest.mark.parametrize("nx,ny", [(96, 80), (128, 256), (2048, 64), (768, 384)])
def test_laplacian_inv_and_cn(ib, lib, dev, O, monkeypatch, nx, ny, dst):
    monkeypatch.setenv("IBGB300_DST", dst)
    prob, s = make(ib, nx, ny, 3)
    g = ogrid(O, prob)
    rng = np.random.default_rng(5)
    b = rng.standard_normal((2,) + g.gshape)
    db, dx = dev.put(b), dev.empty(b.size)
    assert lib.ib_op_laplacian_inv(s.handle, 2, dev.p(db), dev.p(dx)) == 0
    assert rel(dev.get(dx), O.laplacian_inv(b, O.lap_eigs(g), g)) < TOL
    expl, impl = O.cn_multipliers(g, 0.01, 100.0)
    for lev in (1, 2, 3):
        db1, dx1 = dev.put(b[0]), dev.empty(g.ngamma)
        assert lib.ib_op_cn_ainv(s.handle, lev, dev.p(db1), dev.p(dx1)) == 0
        assert rel(dev.get(dx1), O.laplacian_inv(b[0], impl[lev - 1], g)) < TOL
        assert lib.ib_op_cn_a(s.handle, lev, dev.p(db1), dev.p(dx1)) == 0
        assert rel(dev.get(dx1), O.laplacian_inv(b[0], expl[lev - 1], g)) < TOL
    s.close()


def test_stencils(ib, lib, dev, O):
    prob, s = make(ib, 64, 48, 2)
    g = ogrid(O, prob)
    rng = np.random.default_rng(6)
    psi = rng.standard_normal(g.gshape)
    bc = rng.standard_normal(g.nbc)
    q = rng.standard_normal(g.nq)
    dpsi, dbc, dq = dev.put(psi), dev.put(bc), dev.empty(g.nq)
    # curl with and without a ring
    assert lib.ib_op_curl(s.handle, dev.p(dpsi), dev.p(dbc), dev.p(dq)) == 0
    np.testing.assert_array_equal(dev.get(dq), O.curl(psi, bc, g))
    assert lib.ib_op_curl(s.handle, dev.p(dpsi), None, dev.p(dq)) == 0
    np.testing.assert_array_equal(dev.get(dq), O.curl(psi, np.zeros(g.nbc), g))
    # rot
    dq2, dg = dev.put(q), dev.empty(g.ngamma)
    assert lib.ib_op_rot(s.handle, dev.p(dq2), dev.p(dg)) == 0
    np.testing.assert_array_equal(dev.get(dg).reshape(g.gshape), O.rot(q, g))
    # get_bc
    dr, dring = dev.put(psi), dev.empty(g.nbc)
    assert lib.ib_op_get_bc(s.handle, dev.p(dr), dev.p(dring)) == 0
    np.testing.assert_array_equal(dev.get(dring), O.get_bc(psi, g))
    # apply_bc
    r = rng.standard_normal(g.gshape)
    dr2 = dev.put(r)
    assert lib.ib_op_apply_bc(s.handle, dev.p(dr2), dev.p(dbc), 0.37) == 0
    want = r.copy()
    O.apply_bc(want, bc, 0.37, g)
    assert rel(dev.get(dr2), want) < 1e-15
    # coarsify
    gc = rng.standard_normal(g.gshape)
    gf = rng.standard_normal(g.gshape)
    dgc, dgf = dev.put(gc), dev.put(gf)
    assert lib.ib_op_coarsify(s.handle, dev.p(dgc), dev.p(dgf)) == 0
    want = gc.copy()
    O.coarsify(want, gf, g)
    assert rel(dev.get(dgc), want) < 1e-15
    s.close()


@pytest.mark.parametrize("lev", [1, 2])
def test_nonlinear(ib, lib, dev, O, lev):
    prob, s = make(ib, 64, 48, 2)
    g = ogrid(O, prob)
    rng = np.random.default_rng(7 + lev)
    q = rng.standard_normal(g.nq)
    G = rng.standard_normal(g.gshape)
    bc = rng.standard_normal(g.nbc)
    u, v = 0.9, -0.2
    dq, dG, dbc, dn = dev.put(q), dev.put(G), dev.put(bc), dev.empty(g.ngamma)
    assert lib.ib_op_nonlinear(s.handle, lev, dev.p(dq), u, v, dev.p(dG), dev.p(dbc), dev.p(dn)) == 0
    q0 = O.base_flux(g, u, v)[lev - 1]
    want = O.nonlinear(q, q0, G, bc, lev, g)
    assert rel(dev.get(dn), want) < 1e-14
    s.close()


def test_vort2flux(ib, lib, dev, O):
    prob, s = make(ib, 64, 64, 3)
    g = ogrid(O, prob)
    rng = np.random.default_rng(9)
    G = rng.standard_normal((g.nlevels,) + g.gshape)
    dG, dpsi, dq = dev.put(G), dev.empty(G.size), dev.empty(g.nlevels * g.nq)
    assert lib.ib_op_vort2flux(s.handle, dev.p(dG), dev.p(dpsi), dev.p(dq)) == 0
    Gw = G.copy()
    psi, q = O.vort2flux(Gw, g, O.lap_eigs(g))
    assert rel(dev.get(dG), Gw) < 1e-15
    assert rel(dev.get(dpsi), psi) < TOL
    assert rel(dev.get(dq), q) < TOL
    s.close()


def cyl(ib, n, D, c=(0.5, 0.0)):
    t = 2 * np.pi * np.arange(n) / n
    xb = np.stack([c[0] + D / 2 * np.cos(t), c[1] + D / 2 * np.sin(t)], 1)
    return ib.RigidBody(ib.GridFrame(), xb, np.full(n, np.pi * D / n))


def test_regularization_gather_scatter(ib, lib, dev, O):
    body = cyl(ib, 60, 1.0)
    prob, s = make(ib, 96, 64, 2, [body])
    g = ogrid(O, prob)
    reg = O.reg_update(body.xb, g)
    nb = body.npoints()
    bi = np.zeros(2 * nb, dtype=np.int32)
    w = np.zeros(nb * 2 * 169)
    import ctypes
    assert lib.ib_get_reg(s.handle, bi.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                          w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
    np.testing.assert_array_equal(bi.reshape(nb, 2), reg.body_idx)
    assert np.max(np.abs(w.reshape(reg.weight.shape) - reg.weight)) < 1e-15
    rng = np.random.default_rng(10)
    q = rng.standard_normal(g.nq)
    dq, dfb = dev.put(q), dev.empty(2 * nb)
    assert lib.ib_op_reg_gather(s.handle, dev.p(dq), 0.7, 0.1, dev.p(dfb)) == 0
    qq = q + O.base_flux(g, 0.7, 0.1)[0]
    assert rel(dev.get(dfb), O.reg_gather(qq, reg, g)) < 1e-14
    f = rng.standard_normal(2 * nb)
    df, dqo = dev.put(f), dev.empty(g.nq)
    assert lib.ib_op_reg_scatter(s.handle, dev.p(df), dev.p(dqo)) == 0
    assert rel(dev.get(dqo), O.reg_scatter(f, reg, g)) < 1e-14
    s.close()


def test_schur_matrix_and_inverse(ib, lib, O):
    body = cyl(ib, 48, 1.0)
    prob, s = make(ib, 96, 64, 3, [body])
    g = ogrid(O, prob)
    reg = O.reg_update(body.xb, g)
    _, impl = O.cn_multipliers(g, 0.01, 100.0)
    Bref = O.schur_matrix(reg, g, O.lap_eigs(g), impl[0])
    nf = Bref.shape[0]
    B = np.zeros(nf * nf)
    Bi = np.zeros(nf * nf)
    import ctypes
    dp = ctypes.POINTER(ctypes.c_double)
    assert lib.ib_get_schur(s.handle, B.ctypes.data_as(dp), Bi.ctypes.data_as(dp)) == 0
    B = B.reshape(nf, nf).T   # column-major on the device
    Bi = Bi.reshape(nf, nf).T
    assert rel(B, Bref) < 1e-12
    assert rel(Bi, np.linalg.inv(Bref)) < 1e-10
    assert np.max(np.abs(Bi @ B - np.eye(nf))) < 1e-9
    s.close()
