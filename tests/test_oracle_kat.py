"""Known-answer checks that pin the FP64 oracle to the reference's formulas (CPU only).

The reference has no tests or golden vectors; every identity here follows from its own code
(file:line in the oracle docstrings).
"""
import math

import numpy as np
import pytest
from scipy import fft as sfft


def small_grid(O, nx=32, ny=24, L=3):
    return O.Grid(nx, ny, L, -1.0, -0.75, 4.0 / nx)


def test_dst1_is_unnormalised_rodft00_and_involution(O):
    g = small_grid(O)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(g.gshape)
    # RODFT00 of a pure sine mode is (N+1) * delta in each dimension
    n = g.nx
    j = np.arange(1, n)
    for m in (1, 5, n - 1):
        y = sfft.dst(np.sin(np.pi * j * m / n), type=1)
        expect = np.zeros(n - 1)
        expect[m - 1] = n
        assert np.allclose(y, expect, atol=1e-12 * n)
    # applying it twice multiplies by 4 nx ny
    assert np.allclose(O.dst2(O.dst2(x)), 4 * g.nx * g.ny * x, rtol=1e-13, atol=1e-12)


def test_dst_matches_dense_sine_matrix(O):
    g = small_grid(O, 16, 12, 1)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(g.gshape)
    Sx = 2 * np.sin(np.pi * np.outer(np.arange(1, g.nx), np.arange(1, g.nx)) / g.nx)
    Sy = 2 * np.sin(np.pi * np.outer(np.arange(1, g.ny), np.arange(1, g.ny)) / g.ny)
    assert np.allclose(O.dst2(x), Sy @ x @ Sx, rtol=1e-13, atol=1e-12)


def test_laplacian_inverse_of_rot_curl(O):
    """rot(curl(psi)) with a zero ring is the 5-point Laplacian, so LaplacianInv undoes it."""
    g = small_grid(O)
    rng = np.random.default_rng(2)
    psi = rng.standard_normal(g.gshape)
    lap = O.rot(O.curl(psi, np.zeros(g.nbc), g), g)
    assert np.allclose(lap, O.rot(O.curl0(psi, g), g))
    back = O.laplacian_inv(lap, O.lap_eigs(g), g)
    assert np.allclose(back, psi, rtol=1e-12, atol=1e-12)
    # eigenfunction: Lambda * phi
    a, b = 3, 4
    I = np.arange(1, g.nx)[None, :]
    J = np.arange(1, g.ny)[:, None]
    phi = np.sin(np.pi * a * I / g.nx) * np.sin(np.pi * b * J / g.ny)
    lam = O.lap_eigs(g)[b - 1, a - 1]
    assert np.allclose(O.rot(O.curl0(phi, g), g), lam * phi, atol=1e-12)


def test_cn_multipliers_invert_each_other(O):
    g = small_grid(O)
    dt, Re = 0.01, 100.0
    expl, impl = O.cn_multipliers(g, dt, Re)
    lam = O.lap_eigs(g)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(g.gshape)
    for l in range(g.nlevels):
        hc = g.hc(l + 1)
        a = dt / (2 * Re * hc * hc)
        # A = I - a L, Ainv = (I + a L)^-1 with L = rot curl
        Lx = O.rot(O.curl0(x, g), g)
        assert np.allclose(O.laplacian_inv(x, expl[l], g), x - a * Lx, rtol=1e-12, atol=1e-12)
        y = O.laplacian_inv(x, impl[l], g)
        assert np.allclose(y + a * O.rot(O.curl0(y, g), g), x, rtol=1e-12, atol=1e-12)
    assert np.all(lam > 0)


def test_delta_moments_and_support(O):
    """Yang-3 delta: unit sum and zero first moment (to the 10-digit constants), support 3h."""
    h = 0.1
    for off in (0.0, 0.013, 0.05, 0.0999):
        xs = h * np.arange(-6, 7) + off
        w = O.delta_h(xs, 0.0, h)
        assert abs(w.sum() - 1.0) < 1e-8
        assert abs((w * xs).sum()) / h < 1e-8
        assert np.all(w[np.abs(xs) > 3 * h] == 0.0)
    assert O.delta_h(np.array([0.0]), 0.0, 1.0)[0] == pytest.approx(0.6485698427 + 8.0187537413e-2 * math.asin(-math.sqrt(3) / 2)
                                                              - 4.195601852e-2, rel=1e-15)


def test_delta_matches_high_precision_evaluation(O):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    rs = np.array([0.0, 0.3, 0.999, 1.0, 1.5, 1.999, 2.0, 2.7, 3.0])

    def ref(r1):
        r1 = mp.mpf(r1)
        r2, r3, r4 = r1 ** 2, r1 ** 3, r1 ** 4
        s3 = mp.sqrt(3)
        if r1 <= 1:
            a5 = mp.asin(s3 / 2 * (2 * r1 - 1)); a8 = mp.sqrt(1 - 12 * r2 + 12 * r1)
            return (mp.mpf("4.166666667e-2") * r4 + (mp.mpf("-0.1388888889") + mp.mpf("3.472222222e-2") * a8) * r3
                    + (mp.mpf("-7.121664902e-2") - mp.mpf("5.208333333e-2") * a8 + mp.mpf("0.2405626122") * a5) * r2
                    + (mp.mpf("-0.2405626122") * a5 - mp.mpf("0.3792313933") + mp.mpf("0.1012731481") * a8) * r1
                    + mp.mpf("8.0187537413e-2") * a5 - mp.mpf("4.195601852e-2") * a8 + mp.mpf("0.6485698427"))
        if r1 <= 2:
            a6 = mp.asin(s3 / 2 * (-3 + 2 * r1)); a9 = mp.sqrt(-23 + 36 * r1 - 12 * r2)
            return (mp.mpf("-6.25e-2") * r4 + (mp.mpf("0.4861111111") - mp.mpf("1.736111111e-2") * a9) * r3
                    + (mp.mpf("-1.143175026") + mp.mpf("7.8125e-2") * a9 - mp.mpf("0.1202813061") * a6) * r2
                    + (mp.mpf("0.8751991178") + mp.mpf("0.3608439183") * a6 - mp.mpf("0.1548032407") * a9) * r1
                    - mp.mpf("0.2806563809") * a6 + mp.mpf("8.22848104e-3") + mp.mpf("0.1150173611") * a9)
        if r1 <= 3:
            a1 = mp.asin((2 * r1 - 5) / 2 * s3); a7 = mp.sqrt(-71 - 12 * r2 + 60 * r1)
            return (mp.mpf("2.083333333e-2") * r4 + (mp.mpf("3.472222222e-3") * a7 - mp.mpf("0.2638888889")) * r3
                    + (mp.mpf("1.214391675") - mp.mpf("2.604166667e-2") * a7 + mp.mpf("2.405626122e-2") * a1) * r2
                    + (mp.mpf("-0.1202813061") * a1 - mp.mpf("2.449273192") + mp.mpf("7.262731481e-2") * a7) * r1
                    + mp.mpf("0.1523563211") * a1 + mp.mpf("1.843201677") - mp.mpf("7.306134259e-2") * a7)
        return mp.mpf(0)

    got = O.delta_h(rs, 0.0, 1.0)
    want = np.array([float(ref(r)) for r in rs])
    # near r = 3 the O(1) terms cancel to ~1e-9, so FP64 keeps ~1e-15 absolute accuracy there
    assert np.allclose(got, want, rtol=1e-13, atol=1e-14)


def body_setup(O, g, n=40, D=None):
    D = D or 0.3 * (g.nx * g.h)
    t = 2 * np.pi * np.arange(n) / n
    cx = g.x0 + 0.5 * g.nx * g.h
    cy = g.y0 + 0.5 * g.ny * g.h
    return np.stack([cx + D / 2 * np.cos(t), cy + D / 2 * np.sin(t)], 1)


def test_E_and_ET_are_adjoint(O):
    g = small_grid(O, 48, 40, 2)
    xb = body_setup(O, g)
    reg = O.reg_update(xb, g)
    rng = np.random.default_rng(4)
    q = rng.standard_normal(g.nq)
    f = rng.standard_normal(2 * xb.shape[0])
    assert np.dot(O.reg_gather(q, reg, g), f) == pytest.approx(np.dot(q, O.reg_scatter(f, reg, g)), rel=1e-13)


def test_scatter_rejects_nonfinite_and_out_of_grid(O):
    g = small_grid(O, 48, 40, 2)
    xb = body_setup(O, g)
    reg = O.reg_update(xb, g)
    f = np.zeros(2 * xb.shape[0])
    f[3] = np.nan
    with pytest.raises(FloatingPointError):
        O.reg_scatter(f, reg, g)
    bad = xb.copy()
    bad[0] = (g.x0 + 2 * g.h, g.y0 + 0.5 * g.ny * g.h)
    with pytest.raises(IndexError):
        O.reg_gather(np.zeros(g.nq), O.reg_update(bad, g), g)


def test_freestream_invariance(O):
    """No body, Gamma = 0: the nonlinear term vanishes and Gamma stays zero."""
    g = small_grid(O, 32, 32, 2)
    prob = O.Problem(g, 0.01, 100.0, np.zeros((0, 2)), np.zeros(0), [])
    st = O.init_state(prob)
    sol = O.Solver(prob)
    for i in range(3):
        sol.advance(st, i * prob.dt)
    assert np.all(st.gamma == 0.0)
    qx, qy = O.split_flux(st.q[0], g)
    assert np.all(qx == 0.0) and np.all(qy == 0.0)


def test_schur_matrix_nearly_symmetric_positive(O):
    g = small_grid(O, 48, 48, 2)
    xb = body_setup(O, g, 24)
    reg = O.reg_update(xb, g)
    lam = O.lap_eigs(g)
    _, impl = O.cn_multipliers(g, 0.01, 100.0)
    B = O.schur_matrix(reg, g, lam, impl[0], batch=16)
    asym = np.linalg.norm(B - B.T) / np.linalg.norm(B)
    assert asym < 1e-3
    assert np.all(np.linalg.eigvalsh(0.5 * (B + B.T)) > 0)
    # batched assembly equals column-by-column B_times
    e = np.zeros(B.shape[0])
    e[5] = 1.0
    assert np.allclose(O.b_times(e, reg, g, lam, impl[0]), B[:, 5], rtol=1e-13, atol=1e-16)


def test_coarsify_get_bc_apply_bc_index_maps(O):
    """Coarsify writes only the coarse centre; get_bc of a field linear in the coarse node
    index interpolates linearly along the fine edge."""
    g = small_grid(O, 16, 16, 2)
    gc = np.full(g.gshape, 7.0)
    gf = np.ones(g.gshape)
    O.coarsify(gc, gf, g)
    assert np.all(gc[4:11, 4:11] == 4.0)  # 1 + 0.5*4 + 0.25*4
    assert gc[3, 3] == 7.0 and gc[11, 11] == 7.0
    I = np.arange(1, g.nx)[None, :] * np.ones((g.ny - 1, 1))
    bc = O.get_bc(I, g)
    # bottom edge: fine node i (0..nx) sits at coarse node nx/4 + i/2
    i = np.arange(g.nx + 1)
    assert np.allclose(bc[g.B:g.B + g.nx + 1], 0.25 * (g.nx / 4 + i / 2))
    r = np.zeros(g.gshape)
    O.apply_bc(r, bc, 2.0, g)
    assert r[0, 0] == pytest.approx(2.0 * (bc[g.B + 1] + bc[g.L + 1]))


def test_mlp_oracle_gradient_matches_finite_differences():
    """The network oracle's backward pass (float64, unrounded weights) against central
    differences of its loss."""
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(3)
    dims = [7, 5, 6, 4]
    n = sum(dims[i] * dims[i + 1] + dims[i + 1] for i in range(len(dims) - 1))
    p = rng.standard_normal(n) * 0.5
    x = rng.standard_normal((9, dims[0]))
    y = rng.standard_normal((9, dims[-1]))
    loss, g = M.loss_and_grad(p, dims, x, y, bf16=False)
    eps = 1e-6
    fd = np.zeros(n)
    for i in range(n):
        e = np.zeros(n)
        e[i] = eps
        fd[i] = (M.loss_and_grad(p + e, dims, x, y, bf16=False)[0] - M.loss_and_grad(p - e, dims, x, y, bf16=False)[0]) / (2 * eps)
    assert np.max(np.abs(fd - g)) < 1e-7 * max(1.0, np.max(np.abs(g)))
    assert loss > 0


def test_bf16_rounding_is_nearest_even():
    from oracle import mlp_oracle as M
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 3.0e-3], dtype=np.float32)
    r = M.bf16_round(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0 + 2 ** -7)
    assert r[3] == np.float32(1.0 + 2 ** -6)  # tie between 1+2^-7 and 1+2^-6 goes to the even mantissa
    assert r[4] == -2.5
    assert abs(r[5] - 3.0e-3) <= 2 ** -8 * 3.0e-3  # half an ulp of an 8-bit significand


def test_preconditioned_schur_solve_matches_dense_inverse(O):
    """The oracle's iterative Schur solve (used where assembling B is too slow on the CPU)
    reaches the dense inverse's answer whatever preconditioner it is given."""
    g = small_grid(O, 48, 48, 2)
    xb = body_setup(O, g, 24)
    prob = O.Problem(g, 0.01, 100.0, xb, np.full(24, 0.1), [24])
    dense = O.Solver(prob)
    rng = np.random.default_rng(5)
    # a preconditioner 1% away from the inverse, as a neighbouring configuration would give
    P = dense.Binv @ (np.eye(dense.Binv.shape[0]) + 0.01 * rng.standard_normal(dense.Binv.shape) / 7)
    iters = O.Solver(prob, precond=P)
    st0 = O.init_state(prob)
    st0.gamma[0] = 1e-3 * rng.standard_normal(g.gshape)
    st0.psi, st0.q = O.vort2flux(st0.gamma, g, O.lap_eigs(g))
    a, b = st0.copy(), st0.copy()
    for i in range(3):
        dense.advance(a, i * prob.dt)
        iters.advance(b, i * prob.dt)
    assert np.linalg.norm(a.fb - b.fb) / np.linalg.norm(a.fb) < 1e-11
    assert np.linalg.norm(a.gamma - b.gamma) / np.linalg.norm(a.gamma) < 1e-12
    assert 1 <= max(iters.refine_iterations) < 15


def test_checkpoint_format_round_trip(O, tmp_path):
    """The checkpoint layout (header + column-major FP64 arrays) read back field by field;
    files of another grid, a wrong magic or a short body are refused."""
    g = small_grid(O, 32, 24, 3)
    prob = O.Problem(g, 0.01, 100.0, np.zeros((0, 2)), np.zeros(0), [])
    st = O.init_state(prob, 0.37)
    rng = np.random.default_rng(2)
    st.gamma = rng.standard_normal(st.gamma.shape)
    st.psi = rng.standard_normal(st.psi.shape)
    st.q = rng.standard_normal(st.q.shape)
    st.nonlin = [rng.standard_normal(st.gamma.shape), rng.standard_normal(st.gamma.shape)]
    st.fb = rng.standard_normal(6)
    path = tmp_path / "a.ckpt"
    O.write_checkpoint(path, g, st, steps=12, fb_prev=np.arange(6.0))
    raw = path.read_bytes()
    assert raw[:8] == b"IBGB300C" and len(raw) == 56 + 8 * (4 * 3 * g.ngamma + 3 * g.nq + 12)
    ck = O.read_checkpoint(path, g)
    assert ck["t"] == 0.37 and ck["steps"] == 12
    for k in ("gamma", "psi", "q", "fb"):
        np.testing.assert_array_equal(ck[k], getattr(st, k))
    np.testing.assert_array_equal(ck["nonlin"][0], st.nonlin[0])
    np.testing.assert_array_equal(ck["nonlin"][1], st.nonlin[1])
    np.testing.assert_array_equal(ck["fb_prev"], np.arange(6.0))
    with pytest.raises(ValueError):
        O.read_checkpoint(path, small_grid(O, 32, 32, 3))
    bad = tmp_path / "b.ckpt"
    bad.write_bytes(b"XXXXXXXX" + raw[8:])
    with pytest.raises(ValueError):
        O.read_checkpoint(bad, g)
    bad.write_bytes(raw[:-8])
    with pytest.raises(ValueError):
        O.read_checkpoint(bad, g)


def test_rkc_coefficients_and_stability_interval(O):
    """RKC with 2/13 damping: the stability interval grows like s^2 toward the published
    ~0.653 s^2, and the stage coefficients are consistent (exact for dY/dt = 1)."""
    prev = 0.0
    for S in (2, 3, 5, 10, 20):
        mu, nu, mut, gamt, beta = O.rkc_coefficients(S)
        assert 0.45 * S * S < beta < 0.66 * S * S and beta / (S * S) > prev
        prev = beta / (S * S)
        # integrate dy/dt = 1 from 0 over dt = 1: every stage's y equals its stage time c_j,
        # and the last one reaches 1
        y = [0.0, mut[1]]
        for j in range(2, S + 1):
            y.append((1 - mu[j] - nu[j]) * 0.0 + mu[j] * y[j - 1] + nu[j] * y[j - 2] + mut[j] + gamt[j])
        assert abs(y[S] - 1.0) < 1e-12


def test_rkc_is_second_order_in_time(O):
    """No body, smooth vorticity on a 2-level grid: halving dt quarters the error at a fixed time."""
    g = small_grid(O, 32, 32, 2)
    prob0 = O.Problem(g, 0.02, 50.0, np.zeros((0, 2)), np.zeros(0), [], freestream=(0.3, 0.1))
    xs = (np.arange(1, g.nx) - g.nx / 2) / (g.nx / 6)
    ys = (np.arange(1, g.ny) - g.ny / 2) / (g.ny / 6)
    omega = np.exp(-(xs[None, :] ** 2 + ys[:, None] ** 2))

    def run(dt, n):
        prob = O.Problem(g, dt, prob0.Re, prob0.xb, prob0.ds, [], freestream=prob0.freestream)
        st = O.init_state(prob)
        st.gamma[0] = 1e-2 * omega * g.h ** 2
        st.psi, st.q = O.vort2flux(st.gamma, g, O.lap_eigs(g))
        sol = O.RKCSolver(prob, stages=3)
        for i in range(n):
            sol.advance(st, i * dt)
        return st.gamma[0].copy()
    ref = run(0.0025, 32)
    e1 = np.linalg.norm(run(0.02, 4) - ref)
    e2 = np.linalg.norm(run(0.01, 8) - ref)
    e3 = np.linalg.norm(run(0.005, 16) - ref)
    assert 3.0 < e1 / e2 < 5.0 and 3.0 < e2 / e3 < 5.5, (e1, e2, e3)
