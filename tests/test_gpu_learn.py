"""Learned warm start of the moving-body Schur CG (include/ibgb300_learn.h): the device
network's loss and gradients against the float64 oracle, and what the trained network gains
over linear extrapolation on steps it was not trained on."""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def heaving(ib, nx=128, ny=96, L=2, f=0.5, heave=0.25, pitch_deg=15.0, dt=0.005):
    """A plate heaving and pitching at f (period 1/(f dt) = 400 steps); stable at this time step
    (at f = 1 it needs dt = 0.0025: the explicit advection near the plate edges limits dt)."""
    W = ib.workloads
    frame = W.heave_pitch_frame(f=f, heave=heave, pitch_deg=pitch_deg)
    base = W.Workload("heaving_test", 0.005, (-1.0, 2.84), (-1.28, 1.28), L, 200.0, dt, 10,
                      [W.moving_plate(201, frame=frame)])
    wl = W.scaled(base, nx, ny, nlevels=L, nsteps=10)
    wl.Re = 200.0
    wl.dt = dt
    return wl


def test_gradients_match_oracle(ib):
    wl = heaving(ib)
    prob = wl.problem()
    st = ib.initstate(prob)
    s = ib.initsolver(prob, st)
    s.learn_init(hidden=48, layers=3, capacity=16, seed=1)
    dims = s.learn_layout()
    assert dims[0] == 6 + 2 * 2 * s.nb and dims[-1] == 2 * s.nb and dims[1:-1] == [48, 48, 48]
    rng = np.random.default_rng(7)
    p = (0.3 * rng.standard_normal(s.learn_params().size)).astype(np.float32)
    s.learn_params(p)
    np.testing.assert_array_equal(s.learn_params(), p)
    x = rng.standard_normal((37, dims[0])).astype(np.float32)
    y = rng.standard_normal((37, dims[-1])).astype(np.float32)
    loss, g = s.learn_gradients(x, y)
    oloss, og = M.loss_and_grad(p, dims, x, y)
    assert abs(loss - oloss) <= 1e-5 * oloss
    off = 0
    for l in range(len(dims) - 1):
        for n in (dims[l] * dims[l + 1], dims[l + 1]):  # W_l then b_l
            a, b = g[off: off + n], og[off: off + n]
            assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b), (l, n)
            off += n
    assert off == g.size
    s.close()


def run(ib, wl, warm, n_train, n_eval, train_kw, blend=None):
    prob = wl.problem()
    st = ib.initstate(prob)
    s = ib.initsolver(prob, st)
    s.set_cg_options(tol=1e-10, warm_start="extrapolate")
    s.learn_init(hidden=128, layers=3, capacity=1024, seed=0)
    s.learn_collect(True)
    for i in range(n_train):
        ib.advance_(st, s, i * wl.dt)
    loss = None
    if warm == "learned":
        loss = s.learn_train(**train_kw)
        loss = (loss,) + s.learn_validation()
        s.set_cg_options(tol=1e-10, warm_start="learned")
        if blend is not None:
            s.learn_set_blend(blend)
    for i in range(n_train, n_train + n_eval):
        ib.advance_(st, s, i * wl.dt)
    it, res, r0 = s.cg_stats(n_eval, start=True)
    samples = s.learn_samples()
    s.close()
    return it, res, r0, loss, samples


def test_learned_warm_start_converges_and_does_not_regress_on_held_out_steps(ib):
    wl = heaving(ib)
    n_train, n_eval = 500, 40
    kw = dict(epochs=400, batch=32, lr=1e-3, seed=0)
    it_e, res_e, r0_e, _, _ = run(ib, wl, "extrapolate", n_train, n_eval, kw)
    it_l, res_l, r0_l, loss, samples = run(ib, wl, "learned", n_train, n_eval, kw)
    assert samples == n_train + n_eval - 2  # recording continues while the network is used
    # CG decides both: the same tolerance is reached on every step
    assert np.all(res_e <= 1e-10) and np.all(res_l <= 1e-10)
    print(f"loss {loss[0]:.3e} blend {loss[1]:.3f} held-out rel err {loss[2]:.3e}  "
          f"r0 extrapolated {np.mean(r0_e):.3e}  learned {np.mean(r0_l):.3e}  "
          f"iterations {it_e.sum()} -> {it_l.sum()}")
    # the validated blend never makes the start worse than extrapolation on held-out rows
    assert 0.0 <= loss[1] <= 1.0 and loss[2] <= 1.0
    assert np.mean(r0_l) <= 1.05 * np.mean(r0_e)
    assert it_l.sum() <= it_e.sum() * 1.01


def test_zero_blend_start_is_extrapolation_on_the_same_trajectory(ib):
    """With the network's correction weighted 0 the learned arm starts every CG solve exactly
    where the extrapolating arm does (the same start residuals and iteration counts, step by
    step): the learned arm's features and force history belong to the current step, so the
    gap between the two arms' start residuals at the validated blend is the correction
    itself.  That correction minimises the held-out error of F in the 2-norm, while the start
    residual weighs it by B (cond ~1e4-1e5): a small blend of a correction that is rough along
    the plate can still raise ||B x0 - rhs||."""
    wl = heaving(ib)
    n_train, n_eval = 200, 20
    kw = dict(epochs=100, batch=32, lr=1e-3, seed=0)
    it_e, res_e, r0_e, _, _ = run(ib, wl, "extrapolate", n_train, n_eval, kw)
    it_0, res_0, r0_0, _, _ = run(ib, wl, "learned", n_train, n_eval, kw, blend=0.0)
    np.testing.assert_array_equal(r0_0, r0_e)
    np.testing.assert_array_equal(it_0, it_e)


def test_network_export_import_reproduces_the_predictions(ib):
    """A trained network moved to a second handle (ib_learn_export / ib_learn_import) gives that
    handle the same warm starts: both continue the same run to the same bits."""
    wl = heaving(ib)
    arms = []
    for k in range(2):
        prob = wl.problem()
        st = ib.initstate(prob)
        s = ib.initsolver(prob, st)
        s.set_cg_options(tol=1e-10, warm_start="extrapolate")
        s.learn_init(hidden=64, layers=3, capacity=512, seed=0)
        s.learn_collect(True)
        arms.append((st, s))
    for i in range(120):
        for st, s in arms:
            ib.advance_(st, s, i * wl.dt)
    arms[0][1].learn_train(epochs=40, batch=32, lr=1e-3, seed=0)
    arms[0][1].learn_set_blend(0.5)
    buf = arms[0][1].learn_export()
    arms[1][1].learn_import(buf)
    np.testing.assert_array_equal(arms[1][1].learn_export(), buf)
    for st, s in arms:
        s.set_cg_options(tol=1e-10, warm_start="learned")
    for i in range(120, 130):
        for st, s in arms:
            ib.advance_(st, s, i * wl.dt)
    np.testing.assert_array_equal(arms[0][0].qty.Fb, arms[1][0].qty.Fb)
    r0 = [s.cg_stats(10, start=True)[2] for _, s in arms]
    np.testing.assert_array_equal(r0[0], r0[1])
    for _, s in arms:
        s.close()
