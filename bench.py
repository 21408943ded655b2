"""Benchmark of the GB300 CNAB immersed-boundary step (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload NAME]

A step is one ``advance!`` of the workload (every level of the multilevel grid, the Schur
force solve and the projection).  ``value`` is cell-steps/s (cells = nlevels * nx * ny per
step) over all ranks with the state resident on the device; ``e2e`` is the same metric
through the public ``solve`` API with a per-step host callback reading C_D / C_L.  Under
torchrun each rank advances an independent replica on its own GPU (the step has no
data-parallel split).

``--impl reference`` times the CPU implementation of the same step on this host's cores (the
FP64 restatement of the reference; Julia is not available) on the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-steps/s on 1 GB300: learned+mixed vs plain FP64 GPU at C_L/C_D err \u22641e-6"


def baseline_metric() -> str:
    return METRIC


# DRAM bytes (read + write) per launch of each pass class, from an ncu capture of one step of the
# same workload and precision with the kernel choice the bench runs (dram__bytes_read.sum +
# dram__bytes_write.sum over every launch of the class in the step, divided by the launches).
# The summary with the command that made it is under profiles/; its machine-readable lines read
#   traffic <workload> <precision> <form> <class> <bytes per launch> <launches>
TRAFFIC_PROFILE = ROOT / "profiles" / "traffic_two_body_large.md"


def measured_traffic(workload: str, precision: str, form: str, cls: str):
    """(bytes per launch, launches captured, source) from the committed capture, or None."""
    if not TRAFFIC_PROFILE.exists():
        return None
    for line in TRAFFIC_PROFILE.read_text().splitlines():
        f = line.strip().strip("`").split()
        if len(f) == 7 and f[0] == "traffic" and f[1:5] == [workload, precision, form, cls]:
            return float(f[5]), int(f[6]), f"{TRAFFIC_PROFILE.relative_to(ROOT)} (ncu, one step, {f[6]} launches)"
    return None


def measured_issue(workload: str, precision: str, form: str, cls: str):
    """(warp instructions per launch, launches captured, source) from the committed capture, or None."""
    if not TRAFFIC_PROFILE.exists():
        return None
    for line in TRAFFIC_PROFILE.read_text().splitlines():
        f = line.strip().strip("`").split()
        if len(f) == 7 and f[0] == "issue" and f[1:5] == [workload, precision, form, cls]:
            return float(f[5]), int(f[6]), f"{TRAFFIC_PROFILE.relative_to(ROOT)} (ncu smsp__inst_executed.sum, one step, {f[6]} launches)"
    return None


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class Dist:
    """Barrier and max-over-ranks through torch.distributed (only when WORLD_SIZE > 1)."""

    def __init__(self, world: int, local: int, backend: str):
        self.world = world
        self.pg = None
        if world > 1:
            import torch
            import torch.distributed as dist
            if backend == "nccl":
                torch.cuda.set_device(local)
            dist.init_process_group(backend=backend)
            self.dist, self.torch = dist, torch
            self.backend = backend

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = self.torch.tensor([x], dtype=self.torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


def make_workload(ib, name: str):
    w = ib.workloads
    table = {"two_body_large": w.two_body_large, "cylinder_small": w.cylinder_small,
             "four_cylinders": w.four_cylinders, "heaving_plate": w.heaving_plate}
    return table[name]()


# ----------------------------------------------------------------------------------------------
# moving bodies: the plain FP64 GPU path (the reference's algorithm: cg! from the previous Fb, no
# preconditioner) against mixed precision + Schur-preconditioned CG + learned warm start
# ----------------------------------------------------------------------------------------------
def moving_arm(ib, wl, precision, pc, warm, n, timed_from, learn=None):
    prob = wl.problem()
    st = ib.initstate(prob)
    st._gamma[:] = wl.initial_gamma()
    s = ib.initsolver(prob, st, precision=precision)
    s.set_cg_options(tol=1e-10, warm_start="extrapolate" if warm == "learned" else warm)
    s.set_cg_preconditioner(pc)
    s.vort2flux(st)
    info = {}
    if learn:
        s.learn_init(hidden=256, layers=3, capacity=4096, seed=0)
        s.learn_collect(True)
    cd, cl = [], []
    t0 = None
    for i in range(n):
        if learn and i == learn["train_at"]:
            s.lib.ib_synchronize(s.handle)
            a = time.perf_counter()
            loss = s.learn_train(epochs=learn["epochs"], batch=64, lr=1e-3, seed=0)
            blend, rel = s.learn_validation()
            info = {"train_samples": s.learn_samples(), "train_loss": loss, "blend": blend,
                    "held_out_rel_err_vs_extrapolation": rel, "train_s": time.perf_counter() - a}
            s.set_cg_options(tol=1e-10, warm_start="learned")
        if i == timed_from:
            s.lib.ib_synchronize(s.handle)
            t0 = time.perf_counter()
        ib.advance_(st, s, i * wl.dt)
        cd.append([b.CD for b in st.qty.stress])
        cl.append([b.CL for b in st.qty.stress])
    s.lib.ib_synchronize(s.handle)
    sec = (time.perf_counter() - t0) / (n - timed_from)
    it, res, r0 = s.cg_stats(n, start=True)
    pcs = s.cg_preconditioner_stats()
    s.close()
    return dict(sec=sec, it=it, res=res, r0=r0, cd=np.array(cd), cl=np.array(cl), learn=info, pc=pcs)


def run_moving_config(ib, wl, quick=False):
    n_plain = 6 if quick else 12
    plain = moving_arm(ib, wl, "fp64", "none", "previous", n_plain, 2)
    n_train, n_eval = (60, 20) if quick else (300, 60)
    ours = moving_arm(ib, wl, "mixed", "schur_ref", "learned", n_train + n_eval, n_train,
                      learn={"train_at": n_train, "epochs": 200})
    extrap = moving_arm(ib, wl, "mixed", "schur_ref", "extrapolate", n_train + n_eval, n_train)
    m = min(n_plain, len(ours["cd"]))
    err = float(max(np.max(np.abs(ours["cd"][:m] - plain["cd"][:m]) / np.maximum(1, np.abs(plain["cd"][:m]))),
                    np.max(np.abs(ours["cl"][:m] - plain["cl"][:m]) / np.maximum(1, np.abs(plain["cl"][:m])))))
    cells = wl.cells_per_step
    ev = slice(n_train, n_train + n_eval)
    return {
        "workload": describe(wl) + " (moving: heave 0.5 sin(2 pi f t), pitch 30 deg, f=0.2)",
        "value": cells / ours["sec"], "unit": "cell-steps/s", "ms_per_step": ours["sec"] * 1e3,
        "arm": "mixed precision + Schur-preconditioned CG + learned warm start",
        "plain_fp64": {"value": cells / plain["sec"], "ms_per_step": plain["sec"] * 1e3,
                       "arm": "FP64, CG from the previous Fb, no preconditioner (the reference's algorithm)",
                       "steps_timed": n_plain - 2},
        "speedup_vs_plain_fp64": plain["sec"] / ours["sec"],
        "cg_iterations_per_step": {"plain_fp64": float(np.mean(plain["it"][2:])),
                                   "ours_learned": float(np.mean(ours["it"][ev])),
                                   "ours_extrapolated": float(np.mean(extrap["it"][ev]))},
        "cg_start_residual_mean": {"learned": float(np.mean(ours["r0"][ev])),
                                   "extrapolated": float(np.mean(extrap["r0"][ev]))},
        "cg_final_residual_max": float(max(ours["res"].max(), plain["res"].max())),
        "max_cl_cd_err_vs_fp64": err,
        "err_note": f"first {m} steps, |C - C_plain_fp64| / max(1, |C_plain_fp64|), both CG to 1e-10",
        "learned": dict(ours["learn"], eval_steps=n_eval,
                        note="trained on the run's own steps 2..%d, evaluated on the next %d; blend 0 means the "
                             "validated network correction fell back to extrapolation" % (n_train - 1, n_eval)),
        "preconditioner_assemblies": ours["pc"][0],
        "timed_steps": n_eval,
    }


def ensemble_member(ib, w, precision, plain=False):
    prob = w.problem()
    st = ib.initstate(prob)
    st._gamma[:] = w.initial_gamma()
    s = ib.initsolver(prob, st, precision=precision)
    if s.moving:
        if plain:
            s.set_cg_options(tol=1e-10, warm_start="previous")   # the reference's cg! on qty.Fb
        else:
            s.set_cg_options(tol=1e-10, warm_start="extrapolate")
            s.set_cg_preconditioner("schur_ref")
    s.vort2flux(st)
    return st, s


def run_ensemble_config(ib, lib, n=96, K=20, W=3, moving=True):
    """n independent members (with `moving`, every other one pitching) advanced by one graph
    launch per step in mixed precision, against the plain FP64 GPU path stepping the same
    members one at a time (moving ones with the reference's CG: no preconditioner, previous-Fb
    start)."""
    ws = ib.workloads.ensemble(n, moving=moving)
    cells = sum(w.cells_per_step for w in ws)
    a = time.perf_counter()
    runs = [ensemble_member(ib, w, "mixed") for w in ws]
    # moving members take their first two steps on their own (force history, preconditioner);
    # every member does, so that all share the step count
    for w, (st, s) in zip(ws, runs):
        for k in range(2):
            ib.advance_(st, s, k * w.dt)
    setup = time.perf_counter() - a
    ens = ib.Ensemble([s for _, s in runs])
    members, kernels = ens.info()
    times = np.array([[(2 + k) * w.dt for w in ws] for k in range(W + K)])
    ens.advance_n(times[:W], states=[st for st, _ in runs])
    ms = ens.advance_n(times[W:], states=[st for st, _ in runs]) / K
    ens.close()
    iters = [float(np.mean(s.cg_stats(K)[0])) for (st, s) in runs if s.moving]
    iters_max = [int(np.max(s.cg_stats(K)[0])) for (st, s) in runs if s.moving]
    for _, s in runs:
        s.close()
    # plain FP64 GPU path, one member at a time
    t64 = 0.0
    plain_iters = []
    for w in ws:
        st, s = ensemble_member(ib, w, "fp64", plain=True)
        m = 2 if s.moving else 8
        for k in range(2):
            ib.advance_(st, s, k * w.dt)
        lib.ib_synchronize(s.handle)
        a = time.perf_counter()
        if s.moving:
            for k in range(m):
                ib.advance_(st, s, (2 + k) * w.dt)
            lib.ib_synchronize(s.handle)
            t64 += (time.perf_counter() - a) * 1e3 / m
            plain_iters.append(float(np.mean(s.cg_stats(m)[0])))
        else:
            tt = np.ascontiguousarray((2 + np.arange(m)) * w.dt)
            uv = np.ascontiguousarray(np.tile(np.array(w.freestream, dtype=np.float64), m))
            dp = C.POINTER(C.c_double)
            dms = C.c_double()
            s._check(lib.ib_advance_n_timed(s.handle, m, tt.ctypes.data_as(dp), uv.ctypes.data_as(dp),
                                            C.byref(dms)))
            t64 += dms.value / m
        s.close()
    from collections import Counter
    grids = Counter(f"{w.nx}x{w.ny}" for w in ws)
    return {
        "workload": f"ensemble of {members} members ({len(iters)} pitching 15 deg about mid-chord at f=U[0.1,0.3]): "
                    f"grids {dict(grids)}, 3-5 levels, ellipses (aspect U[0.1,1], angle U[0,40] deg, points ~h), "
                    "Re log-uniform [50,500], dt=0.2h",
        "value": cells / (ms / 1e3), "unit": "cell-steps/s", "ms_per_step": ms,
        "arm": "mixed precision, all members in one CUDA graph launch per step (moving members: "
               "Schur-preconditioned CG loop inside the graph)",
        "kernels_per_launch": kernels, "setup_s": setup,
        "cg_iterations_per_step_moving": float(np.mean(iters)) if iters else None,
        "cg_iterations_max_member": max(iters_max) if iters_max else None,
        "note": "members step in lockstep: a step lasts as long as its slowest member's CG",
        "plain_fp64": {"value": cells / (t64 / 1e3), "ms_per_step": t64,
                       "arm": "FP64, one member at a time (moving: plain CG from the previous Fb)",
                       "cg_iterations_per_step_moving": float(np.mean(plain_iters)) if plain_iters else None},
        "speedup_vs_plain_fp64": t64 / ms, "steps": K,
    }


def run_learned_protocol(ib, n_train=2000, n_eval=2000, f_train=0.2, f_unseen=(0.15, 0.25)):
    """The learned warm start under the moving-plate protocol: the network trains on the
    solver's own force history of steps 0..n_train-1 at f_train, then starts the CG solves of
    steps n_train..n_train+n_eval-1 and, carried over to other handles, the solves of
    n_eval steps at each unseen frequency; against linear extrapolation on the same steps.
    Mixed precision, Schur-preconditioned CG to 1e-10 with a fixed re-assembly period (20 steps)
    so that both arms see the same preconditioners."""
    W = ib.workloads

    def arm(f, nsteps, learned, train_at=None, import_buf=None):
        wl = W.heaving_plate(nsteps=nsteps, f=f)
        prob = wl.problem()
        st = ib.initstate(prob)
        st._gamma[:] = wl.initial_gamma()
        s = ib.initsolver(prob, st, precision="mixed")
        s.set_cg_options(tol=1e-10, warm_start="extrapolate")
        s.set_cg_preconditioner("schur_ref", refresh_steps=20)
        s.vort2flux(st)
        info = {}
        if learned:
            s.learn_init(hidden=256, layers=3, capacity=4096, seed=0)
            if import_buf is not None:
                s.learn_import(import_buf)
                s.set_cg_options(tol=1e-10, warm_start="learned")
            else:
                s.learn_collect(True)
        ts = [i * wl.dt for i in range(nsteps)]
        t0 = time.perf_counter()
        if train_at is not None:
            s.advance_n(st, ts[:train_at])
            a = time.perf_counter()
            loss = s.learn_train(epochs=200, batch=64, lr=1e-3, seed=0)
            blend, rel = s.learn_validation()
            info = {"train_samples": s.learn_samples(), "train_loss": loss, "blend": blend,
                    "held_out_rel_err_vs_extrapolation": rel, "train_s": time.perf_counter() - a}
            s.learn_collect(False)
            s.set_cg_options(tol=1e-10, warm_start="learned")
            s.advance_n(st, ts[train_at:])
        else:
            s.advance_n(st, ts)
        sec = time.perf_counter() - t0
        it, res, r0 = s.cg_stats(nsteps, start=True)
        buf = s.learn_export() if (learned and train_at is not None) else None
        s.close()
        return dict(it=np.asarray(it), res=np.asarray(res), r0=np.asarray(r0), info=info, buf=buf, sec=sec)

    def summ(a, sl):
        return {"cg_iterations_mean": float(np.mean(a["it"][sl])), "cg_iterations_max": int(np.max(a["it"][sl])),
                "start_residual_mean": float(np.mean(a["r0"][sl])), "final_residual_max": float(np.max(a["res"][sl]))}
    n = n_train + n_eval
    lrn = arm(f_train, n, True, train_at=n_train)
    ext = arm(f_train, n, False)
    ev = slice(n_train, n)
    out = {"workload": "heaving_plate 768x512x4, Re 1000, dt 0.0005, 201 points, heave 0.5 sin(2 pi f t), "
                       "pitch 30 deg",
           "training": lrn["info"],
           "f_%g_steps_%d_%d" % (f_train, n_train, n): {"learned": summ(lrn, ev), "extrapolated": summ(ext, ev)}}
    for f in f_unseen:
        key = "f_%g_unseen_steps_0_%d" % (f, n_eval)
        sl = slice(2, n_eval)
        res = {}
        for name, learned in (("learned", True), ("extrapolated", False)):
            try:
                a = arm(f, n_eval, learned, import_buf=lrn["buf"] if learned else None)
                res[name] = summ(a, sl)
            except Exception as e:  # reported, not fatal: the other arms still run
                res[name] = {"error": str(e)}
        out[key] = res
    return out


def run_dt_probe(ib, dt=0.001, nsteps=40):
    """Largest |Gamma| on the finest level per step of the moving plate at a given time step
    (FP64 path, CG to 1e-10): the growth factor shows whether the step is stable."""
    wl = ib.workloads.heaving_plate(nsteps=nsteps, dt=dt)
    prob = wl.problem()
    st = ib.initstate(prob)
    st._gamma[:] = wl.initial_gamma()
    s = ib.initsolver(prob, st, precision="fp64")
    s.set_cg_options(tol=1e-10, warm_start="previous")
    s.set_cg_preconditioner("schur_ref")
    s.vort2flux(st)
    gmax, err = [], None
    try:
        for i in range(nsteps):
            ib.advance_(st, s, i * wl.dt)
            gmax.append(float(np.max(np.abs(st.qty.gamma[0]))))
    except Exception as e:  # a blown-up state ends the run with the library's status
        err = str(e)
    s.close()
    g = np.array(gmax)
    return {"dt": dt, "steps_run": len(gmax), "gamma_max": gmax,
            "growth_per_step_last5": [float(x) for x in (g[-5:] / g[-6:-1])] if g.size > 6 else None,
            "stopped_by": err}


def _device_ms_per_step(ib, s, prob, dt, first, K, W=5):
    """Device milliseconds per step of K captured-graph replays (CUDA events on the handle's
    stream, ib_advance_n_timed) after W warm-up steps, from step index `first`."""
    ts = (first + np.arange(W + K)) * dt
    uv = np.array([prob.fluid.grid_flow(float(t)) for t in ts], dtype=np.float64).reshape(-1)
    dp = C.POINTER(C.c_double)
    tw, uw = np.ascontiguousarray(ts[:W]), np.ascontiguousarray(uv[:2 * W])
    tk, uk = np.ascontiguousarray(ts[W:]), np.ascontiguousarray(uv[2 * W:])
    s._check(s.lib.ib_advance_n(s.handle, W, tw.ctypes.data_as(dp), uw.ctypes.data_as(dp)))
    ms = C.c_double()
    s._check(s.lib.ib_advance_n_timed(s.handle, K, tk.ctypes.data_as(dp), uk.ctypes.data_as(dp), C.byref(ms)))
    return ms.value / K


def run_next_rows(ib, K=20):
    """Measurements of the rows either side of the step on the 1024^2 x 4 two-body workload:
    SchemeRKC against CNAB (FP64), a translating grid frame against the lab frame (mixed),
    checkpoint write / read throughput, and solve_ with sparse (at_indices) callbacks, whose
    steps in between run as graph-replay batches, against a per-step callback."""
    wl = make_workload(ib, "two_body_large")
    cells = wl.cells_per_step
    out = {"workload": describe(wl)}

    def start(prob, precision):
        st = ib.initstate(prob)
        st._gamma[:] = wl.initial_gamma()
        s = ib.initsolver(prob, st, precision=precision)
        s.vort2flux(st)
        return st, s

    disc = ib.MultiLevel(ib.UniformGrid(wl.h, wl.xlims, wl.ylims), wl.nlevels)
    fs = wl.freestream
    # SchemeRKC vs SchemeCNAB, FP64
    rk = {}
    for name, scheme in (("cnab", ib.SchemeCNAB(wl.dt)), ("rkc", ib.SchemeRKC(wl.dt))):
        prob = ib.Problem(ib.StreamFcnFluid(disc, lambda t: fs, wl.Re), ib.BodyGroup(*wl.bodies), scheme)
        st, s = start(prob, "fp64")
        from ibgb300 import _lib as L
        info = L.IbInfo()
        s._check(s.lib.ib_get_info(s.handle, C.byref(info)))
        ms = _device_ms_per_step(ib, s, prob, wl.dt, 0, K)
        rk[name] = {"ms_per_step": ms, "cell_steps_per_s": cells / (ms / 1e3), "kernels_per_step": info.kernels_per_step}
        if name == "rkc":
            rk[name]["stages"] = info.rkc_stages
        s.close()
    out["scheme_rkc_fp64"] = rk
    # translating grid (RelativeFrame of the lab frame) vs lab frame, mixed
    mg = {}
    frame = ib.RelativeFrame(ib.LabFrame(), r=lambda t: (-0.5 * t, 0.0), v=lambda t: (-0.5, 0.0),
                             theta=lambda t: 0.0, omega=lambda t: 0.0)
    for name, dom in (("lab", disc), ("translating", ib.FluidDomain(disc, frame))):
        prob = ib.Problem(ib.StreamFcnFluid(dom, lambda t: fs, wl.Re), ib.BodyGroup(*wl.bodies), ib.SchemeCNAB(wl.dt))
        st, s = start(prob, "mixed")
        ms = _device_ms_per_step(ib, s, prob, wl.dt, 0, K)
        mg[name] = {"ms_per_step": ms, "grid_flow_t0": list(prob.fluid.grid_flow(0.0))}
        s.close()
    out["moving_grid_mixed"] = mg
    # checkpoint files
    prob = wl.problem()
    st, s = start(prob, "mixed")
    for i in range(3):
        ib.advance_(st, s, i * wl.dt)
    path = os.path.join(tempfile.gettempdir(), f"ibgb300_bench_{os.getpid()}.ckpt")
    try:
        a = time.perf_counter()
        s.save_checkpoint(path)
        t_save = time.perf_counter() - a
        nbytes = os.path.getsize(path)
        a = time.perf_counter()
        s.load_checkpoint(path, st)
        t_load = time.perf_counter() - a
    finally:
        if os.path.exists(path):
            os.remove(path)
    out["checkpoint"] = {"bytes": nbytes, "save_s": t_save, "load_s": t_load,
                         "save_gbs": nbytes / t_save / 1e9, "load_gbs": nbytes / t_load / 1e9,
                         "note": "host file in the system temp directory; device state <-> host copies included"}
    s.close()
    # solve_ with callbacks: per-step vs sparse (steps between firings batched)
    cb = {}
    n = 201
    for name, calls in (("each_timestep", lambda: (ib.each_timestep(lambda st_: st_.qty.stress[0].CD),)),
                        ("at_indices_every_50", lambda: (ib.at_indices(lambda st_: st_.qty.stress[0].CD,
                                                                        list(range(1, n + 1, 50))),)),
                        ("none", lambda: ())):
        prob = wl.problem()
        st, s = start(prob, "mixed")
        ib.solve_(st, prob, (0.0, 9 * wl.dt), save=calls(), solver=s)  # warm-up
        s.lib.ib_synchronize(s.handle)
        a = time.perf_counter()
        res = ib.solve_(st, prob, (10 * wl.dt, (10 + n - 1) * wl.dt), save=calls(), solver=s)
        s.lib.ib_synchronize(s.handle)
        sec = (time.perf_counter() - a) / n
        cb[name] = {"ms_per_step": sec * 1e3, "cell_steps_per_s": cells / sec,
                    "samples": len(res[0]) if res else 0}
        s.close()
    out["solve_callbacks_mixed"] = cb
    return out


def run_precision_table(ib, wl, checkpoints=(100, 1000, 2000)):
    """Error of the mixed-precision solve against the FP64 GPU path at the given steps, with the
    sine transforms in FP32 (warp-per-line FFT passes) and as BF16x3 tensor-core GEMMs: relative
    L2 of the vorticity (circulation) and streamfunction over all levels, and the largest C_D /
    C_L error of any body over the steps so far (relative to max(1, |C|))."""
    arms = (("fp64", "fp64", {}), ("fp32", "mixed", {"IBGB300_DST": "warp"}), ("bf16x3", "mixed_tc", {}))
    res = {}
    for name, prec, env in arms:
        old = {k: os.environ.get(k) for k in env}
        os.environ.update(env)
        try:
            prob = wl.problem()
            st = ib.initstate(prob)
            st._gamma[:] = wl.initial_gamma()
            s = ib.initsolver(prob, st, precision=prec, history_capacity=max(checkpoints) + 8)
        finally:
            for k, v in old.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        s.vort2flux(st)
        done, snaps, t0 = 0, {}, time.perf_counter()
        for cp in checkpoints:
            s.advance_n(st, [i * wl.dt for i in range(done, cp)])
            done = cp
            cd, cl = s.force_history(cp)
            snaps[cp] = (st.qty.gamma.copy(), st.qty.psi.copy(), cd, cl)
        res[name] = (snaps, (time.perf_counter() - t0) / max(checkpoints))
        s.close()

    def rl2(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))
    table = {}
    for name in ("fp32", "bf16x3"):
        rows = {}
        for cp in checkpoints:
            g, p, cd, cl = res[name][0][cp]
            g0, p0, cd0, cl0 = res["fp64"][0][cp]
            cerr = max(float(np.max(np.abs(cd - cd0) / np.maximum(1.0, np.abs(cd0)))),
                       float(np.max(np.abs(cl - cl0) / np.maximum(1.0, np.abs(cl0)))))
            rows[str(cp)] = {"omega_rel_l2": rl2(g, g0), "psi_rel_l2": rl2(p, p0), "cl_cd_err_max": cerr}
        table[name] = rows
    return {"workload": describe(wl), "reference_arm": "FP64 GPU path (FP64 sine transforms)",
            "errors": table, "host_s_per_step": {k: v[1] for k, v in res.items()}}


def run_static_config(ib, lib, L, wl, K, W, local, dist):
    arm = run_arm(ib, lib, L, wl, "mixed", K, W, local, dist)
    ref = run_arm(ib, lib, L, wl, "fp64", K, W, local, dist)
    t, t64 = arm["dev_s"], ref["dev_s"]
    err = max(float(np.max(np.abs(arm["cd"] - ref["cd"]) / np.maximum(1.0, np.abs(ref["cd"])))),
              float(np.max(np.abs(arm["cl"] - ref["cl"]) / np.maximum(1.0, np.abs(ref["cl"])))))
    out = {"workload": describe(wl), "value": wl.cells_per_step * K / t, "unit": "cell-steps/s",
           "ms_per_step": t / K * 1e3, "plain_fp64": {"value": wl.cells_per_step * K / t64, "ms_per_step": t64 / K * 1e3},
           "speedup_vs_plain_fp64": t64 / t, "max_cl_cd_err_vs_fp64": err, "steps": K}
    arm["solver"].close()
    ref["solver"].close()
    return out


def bench_config(wl) -> dict:
    """The workload both arms (GPU and CPU reference) report under ``config``; what differs
    between the arms goes under ``arm``."""
    return {"workload": describe(wl), "cells_per_step": wl.cells_per_step,
            "l2": "inputs larger than L2: the per-step working set (state, history, transforms) "
                  "exceeds the 129 MB L2 on every configuration timed"}


def describe(wl) -> str:
    bodies = ", ".join(f"{b.npoints()} pts" for b in wl.bodies)
    return (f"{wl.name}: {wl.nx}x{wl.ny} finest grid h={wl.h}, {wl.nlevels} levels, bodies [{bodies}], "
            f"Re={wl.Re:g}, dt={wl.dt:g}, CNAB")


# ----------------------------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"ibgb300_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.device)], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        try:
            self.path.unlink()
        except Exception:
            pass
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].replace(".", "").isdigit()), default=None)}


# ----------------------------------------------------------------------------------------------
# CPU baseline: the FP64 restatement of the reference on this host's cores
# ----------------------------------------------------------------------------------------------
def cpu_reference(ib, wl, nsteps: int, warmup: int):
    from oracle import ib_oracle as O
    cores = os.cpu_count() or 1
    O.WORKERS = cores
    g = O.grid_from_limits(wl.h, wl.xlims, wl.ylims, wl.nlevels)
    bodies = wl.bodies
    xb = np.concatenate([b.xb for b in bodies])
    ds = np.concatenate([b.ds for b in bodies])
    op = O.Problem(g, wl.dt, wl.Re, xb, ds, [b.npoints() for b in bodies], freestream=wl.freestream)
    st = O.init_state(op)
    st.gamma[0] = wl.initial_gamma()[0].reshape(g.gshape)
    st.psi, st.q = O.vort2flux(st.gamma, g, O.lap_eigs(g))
    sol = O.Solver(op, assemble=False)
    for i in range(warmup):
        sol.advance(st, i * wl.dt)
    t0 = time.perf_counter()
    for i in range(nsteps):
        sol.advance(st, (warmup + i) * wl.dt)
    dt = time.perf_counter() - t0
    return wl.cells_per_step * nsteps / dt, dt / nsteps, cores


# ----------------------------------------------------------------------------------------------
# algorithmic bytes / flops of the sine-transform passes (per step)
# ----------------------------------------------------------------------------------------------
def algorithmic_step_bytes(wl, precision: str) -> float:
    """Compulsory DRAM bytes of one step: w L (5 nGamma + 2 nq) + 8 nf^2 (read Gamma, q and the
    previous nonlinear term, write Gamma, q, psi and the new nonlinear term on every level, read
    the dense Schur inverse once); w = 8 (FP64 values, or float-float pairs)."""
    nG = (wl.nx - 1) * (wl.ny - 1)
    nq = (wl.nx + 1) * wl.ny + wl.nx * (wl.ny + 1)
    nf = 2 * sum(b.npoints() for b in wl.bodies)
    return 8.0 * wl.nlevels * (5 * nG + 2 * nq) + 8.0 * nf * nf


def pass_model(wl, precision: str, levels: bool = False):
    """Algorithmic DRAM bytes and flops of the x and y passes of one step (per step; the bytes per
    launch follow from the launches counted while timing).

    FP64 (every solve one forward and one inverse transform per axis): arrays = the trial CN
    solve over L levels + 2L Vort2Flux solves + the projection; x forward 8 in + 8 out, x inverse
    8 + 8 (+8 for the subtracted trial Gamma), y 8 in + 8 multiplier + 8 out, per element.
    Mixed (default sweep policy): two-sweep solves (CN over L levels, Vort2Flux levels 1-2 twice,
    projection) move per element in x 12 (float-float in, FP32 out) + 8 + 24 (residual: b, x0,
    the stored float-float r1, out) + 8 + 16 (r1, x1, out) + 20 (x0, x1, correction, float-float
    out) and in y 3 x 12; one-sweep solves (Vort2Flux levels 3.. twice) 12 + 8 + 16 + 16 in x and
    2 x 12 in y.  A length-n sine line costs ~2.5 n log2 n flops.
    With the all-levels Vort2Flux (`levels`): the CN and projection solves as above, and per
    Vort2Flux call on every level x 28 (residual from the previous psi: Gamma, psi, r1 out, FP32
    out) + 8 + 24 (residual of x0 on r1, in place) and y 12 + 12 (solve, spectrum), then on the
    finished levels (all, or level 1 for the trial call) x 8 + 16 + 28 (psi += x0 + d1 + d2, read
    and written) and y 12 + 12; 3 + 3 transforms per level in each axis.
    Per class: (bytes, flops, array-passes: one array through one pass).
    """
    nG = (wl.nx - 1) * (wl.ny - 1)
    L = wl.nlevels
    fx = 2.5 * wl.nx * np.log2(wl.nx) * (wl.ny - 1)
    fy = 2.5 * wl.ny * np.log2(wl.ny) * (wl.nx - 1)
    if precision == "fp64":
        arrays = 3 * L + 1
        return {"x": (nG * (32 * arrays + 8), fx * 2 * arrays, 2 * arrays),
                "y": (nG * 24 * arrays, fy * 2 * arrays, arrays)}
    if levels:
        two = L + 1                     # two-sweep CN solves: trial over L levels, projection
        fin = L + 1                     # finished Vort2Flux levels: all (projection) + level 1 (trial)
        xp = 6 * two + 3 * 2 * L + 3 * fin
        return {"x": (nG * (88 * two + 8 + 60 * 2 * L + 52 * fin), fx * xp, xp),
                "y": (nG * (36 * two + 24 * 2 * L + 24 * fin), fy * (6 * two + 3 * 2 * L + 3 * fin),
                      3 * two + 2 * 2 * L + 2 * fin)}
    two, one = L + 5, 2 * max(L - 2, 0)
    return {"x": (nG * (88 * two + 8 + 52 * one), fx * (6 * two + 4 * one), 6 * two + 4 * one),
            "y": (nG * (36 * two + 24 * one), fy * (6 * two + 4 * one), 3 * two + 2 * one)}


def run_arm(ib, lib, L, wl, precision, K, W, local, dist, profile_range=False, refine=0):
    """Set up one solver and time K steps (after W warm-up steps) with CUDA events."""
    prob = wl.problem()
    st = ib.initstate(prob)
    st._gamma[:] = wl.initial_gamma()
    solver = ib.initsolver(prob, st, device=local, precision=precision, refine_sweeps=refine)
    solver.vort2flux(st)
    info = L.IbInfo()
    lib.ib_get_info(solver.handle, C.byref(info))
    n = W + K + 64
    ts = np.ascontiguousarray(np.arange(n, dtype=np.float64) * wl.dt)
    uv = np.ascontiguousarray(np.tile(np.array(wl.freestream, dtype=np.float64), n))

    def tp(a, off):
        return a[off:].ctypes.data_as(C.POINTER(C.c_double))

    solver._check(lib.ib_advance_n(solver.handle, W, tp(ts, 0), tp(uv, 0)))
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    dist.barrier()
    lib.ib_synchronize(solver.handle)
    if profile_range:
        lib.ib_profiler_start()
    dev_ms = C.c_double()
    h0 = time.perf_counter()
    solver._check(lib.ib_advance_n_timed(solver.handle, K, tp(ts, W), tp(uv, 2 * W), C.byref(dev_ms)))
    host_s = time.perf_counter() - h0
    if profile_range:
        lib.ib_profiler_stop()
    dist.barrier()
    ck = clocks.stop()
    cd, cl = solver.force_history(K)
    return dict(solver=solver, state=st, prob=prob, info=info, ts=ts, uv=uv, tp=tp, dev_s=dev_ms.value / 1e3,
                host_s=host_s, clocks=ck, cd=cd, cl=cl)


def run_ours(args, rank, world, local):
    import __graft_entry__ as ge
    ib = ge.package()
    ge.build()
    lib = ib.load_library()
    from ibgb300 import _lib as L
    dist = Dist(world, local, "nccl")
    wl = make_workload(ib, args.workload)
    K, W = args.steps, args.warmup
    prec = args.precision
    arm = run_arm(ib, lib, L, wl, prec, K, W, local, dist, args.profile_range, args.refine_sweeps)
    t_max = dist.max(arm["dev_s"])
    info = arm["info"]
    value = wl.cells_per_step * K * world / t_max
    ms_per_step = t_max / K * 1e3
    out = {
        "metric": baseline_metric(), "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if prec == "fp64" else "f32 transforms + float-float (2xf32) residual/state",
        "data": "synthetic: seeded PCG64 vorticity noise 1e-4 on the finest level",
        "config": bench_config(wl),
        "arm": {"precision": prec,
                "refine_sweeps": (("2 on every solve" if info.vort2flux_order == L.IB_V2F_LEVELS else
                                   {0: "2 (1 on levels >= 3 of Vort2Flux)"}.get(args.refine_sweeps, args.refine_sweeps))
                                  if prec == "mixed" else 0),
                "vort2flux": ("all levels in one batch, rings first (harmonic ring transfer)"
                              if info.vort2flux_order == L.IB_V2F_LEVELS else "level by level (the reference's order)"),
                "parallelism": "replicas",
                "transforms": {0: "Stockham FFT passes", 1: "warp-per-line FFT passes",
                               2: "BF16x3 tensor-core sine GEMMs"}.get(int(info.transform_form)),
                "autotune": arm["solver"].autotune(),
                "device_bytes": int(info.device_bytes),
                "setup_s": info.setup_ms / 1e3, "host_wall_ms_per_step": arm["host_s"] / K * 1e3},
        "gpu_launches": int(info.kernels_per_step) * K,
    }
    ck = arm["clocks"]
    if ck:
        out["clocks"] = {"sm_mhz": ck["sm_mhz"], "sm_max_mhz": ck["sm_max_mhz"], "reasons": ck["reasons"],
                         "samples": ck["samples"], "power_w_max": ck["power_w_max"]}
    if args.profile_range:
        arm["solver"].close()
        print(json.dumps(out), flush=True)
        return
    solver, st, prob, ts, uv, tp = arm["solver"], arm["state"], arm["prob"], arm["ts"], arm["uv"], arm["tp"]
    # dominant kernel class: event-timed launches over further steps
    model = pass_model(wl, prec, levels=prec == "mixed" and info.vort2flux_order == L.IB_V2F_LEVELS)
    prof = {}
    npf = min(K, 20)
    base = W + K
    for cls, key in ((0, "x"), (1, "y")):
        tot, nl = C.c_double(), C.c_int64()
        solver._check(lib.ib_profile_steps(solver.handle, npf, tp(ts, base), tp(uv, 2 * base), cls,
                                           C.byref(tot), C.byref(nl)))
        base += npf
        prof[key] = (tot.value, nl.value)
    dom = max(prof, key=lambda k: prof[k][0])
    tot_ms, nlaunch = prof[dom]
    b_step, f_step, _ = model[dom]
    per_launch_s = tot_ms / 1e3 / nlaunch
    launches_per_step = nlaunch / npf
    bytes_per_launch = b_step / launches_per_step
    flops_per_launch = f_step / launches_per_step
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    fp64, fp32 = C.c_double(), C.c_double()
    lib.ib_measure_fp_peaks(local, C.byref(fp64), C.byref(fp32))
    achieved = bytes_per_launch / per_launch_s / 1e9
    form = {0: "stockham", 1: "warp", 2: "tensor"}.get(int(info.transform_form), "stockham")
    v2f = "levels" if info.vort2flux_order == L.IB_V2F_LEVELS else "sequential"
    meas = measured_traffic(args.workload, prec, f"{form}/{v2f}", dom)
    traffic = meas[0] if meas else None
    pipe_peak = fp64.value if prec == "fp64" else fp32.value
    step_bytes = algorithmic_step_bytes(wl, prec)
    out["roofline"] = {
        "kernel": {"warp": {"x": "k_wxf/k_wxi (x-direction sine passes, one warp per line)",
                            "y": "k_wy (y-direction sine passes + spectral op, one warp per column)"},
                   "stockham": {"x": "k_xpass (x-direction sine pass)",
                                "y": "k_ypass (y-direction sine pass + spectral op)"},
                   "tensor": {"x": "k_gpro + k_sgemm (x-direction BF16x3 sine GEMMs)",
                              "y": "k_sgemm (y-direction BF16x3 sine GEMMs)"}}[form][dom],
        "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6.8 TB/s",
        "traffic": traffic, "algorithmic_bytes_per_launch": bytes_per_launch,
        "traffic_source": meas[2] if meas else None,
        "traffic_frac": (traffic / per_launch_s / 1e9 / hbm) if traffic else None,
        "step": {"algorithmic_bytes": step_bytes, "achieved_gbs": step_bytes / (ms_per_step / 1e3) / 1e9,
                 "frac": step_bytes / (ms_per_step / 1e3) / 1e9 / hbm,
                 "note": "w L (5 nGamma + 2 nq) + 8 nf^2 per step (w = 8 bytes per value: FP64, or a "
                         "float-float pair) over the device time of a step"},
        "avg_launch_ms": per_launch_s * 1e3, "launches_profiled": nlaunch,
        "share_of_step": tot_ms / npf / ms_per_step,
        "fp_pipe": {"pipe": "fp64" if prec == "fp64" else "fp32",
                    "achieved_tflops": flops_per_launch / per_launch_s / 1e12, "peak_tflops": pipe_peak,
                    "frac": flops_per_launch / per_launch_s / 1e12 / pipe_peak if pipe_peak > 0 else None,
                    "peak_source": "measured FMA-chain probe on this GPU"},
        "passes": {k: {"total_ms": prof[k][0], "launches": prof[k][1]} for k in prof},
    }
    # the same launches against the instruction-issue rate: warp instructions per launch (ncu
    # count of these kernels) over 4 schedulers x SMs x SM clock x the event-timed launch
    iss = measured_issue(args.workload, prec, f"{form}/{v2f}", dom)
    if iss and info.sm_count > 0:
        clk = (out.get("clocks") or {}).get("sm_mhz") or (out.get("clocks") or {}).get("sm_max_mhz") or 0.0
        if clk:
            issue_peak = 4.0 * info.sm_count * clk * 1e6
            out["roofline"]["issue"] = {
                "warp_instructions_per_launch": iss[0], "achieved_per_s": iss[0] / per_launch_s,
                "peak_per_s": issue_peak, "frac": iss[0] / per_launch_s / issue_peak,
                "source": iss[2], "note": "one warp instruction per scheduler per cycle; 4 schedulers per SM"}
    # the plain FP64 GPU path on the same workload, and the mixed path's C_L/C_D error against it
    if prec != "fp64" and not args.no_fp64_arm:
        ref = run_arm(ib, lib, L, wl, "fp64", K, W, local, dist)
        t64 = dist.max(ref["dev_s"])
        err = max(float(np.max(np.abs(arm["cd"] - ref["cd"]) / np.maximum(1.0, np.abs(ref["cd"])))),
                  float(np.max(np.abs(arm["cl"] - ref["cl"]) / np.maximum(1.0, np.abs(ref["cl"])))))
        out["fp64_gpu"] = {"value": wl.cells_per_step * K * world / t64, "ms_per_step": t64 / K * 1e3,
                           "speedup_of_headline": t64 / t_max,
                           "max_cl_cd_err_vs_fp64": err,
                           "err_note": f"max over the {K} timed steps and all bodies of |C - C_fp64| / max(1, |C_fp64|)"}
        ref["solver"].close()
    # end to end through the public API: solve_ with a per-step callback reading C_D / C_L
    nb = solver.nb
    t0 = float(ts[base])
    cbs = (ib.each_timestep(lambda s: [(b.CD, b.CL) for b in s.qty.stress]),)
    dist.barrier()
    e0 = time.perf_counter()
    res = ib.solve_(st, prob, (t0, t0 + (K - 1) * wl.dt), save=cbs, solver=solver)
    e2e_s = dist.max(time.perf_counter() - e0)
    assert len(res[0]) == K
    out["e2e"] = {"value": wl.cells_per_step * K * world / e2e_s, "unit": "cell-steps/s",
                  "h2d_bytes_per_step": 8 * 2 * wl.nlevels,
                  "d2h_bytes_per_step": 4 * 3 + 8 * 2 * solver.nbodies + 8 * 2 * nb,
                  "api": "solve_(state, prob, (t0, tf); save=(each_timestep(C_D, C_L),)) per-step advance!"}
    # the other benchmark configurations, one summary each (single-GPU runs; --no-configs skips)
    if world == 1 and not args.no_configs:
        out["configs"] = {
            "four_cylinders": run_static_config(ib, lib, L, ib.workloads.four_cylinders(), 60, 3, local, dist),
            "heaving_plate": run_moving_config(ib, ib.workloads.heaving_plate()),
            "ensemble": run_ensemble_config(ib, lib, K=10, W=2),
            "ensemble_static": run_ensemble_config(ib, lib, K=20, W=3, moving=False),
        }
    if rank == 0 and not args.no_cpu_baseline:
        v, sec, cores = cpu_reference(ib, wl, args.cpu_steps, 1)
        out["cpu_baseline"] = {"value": v, "unit": "cell-steps/s", "cores": cores, "kind": "port",
                               "sample": f"{args.cpu_steps} advance! steps of the same workload at full size "
                                         f"({sec:.2f} s/step; FP64 NumPy/SciPy restatement, scipy.fft workers="
                                         f"{cores}; setup excluded, Schur inverse replaced by a same-size matrix)"}
    solver.close()
    dist.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_reference(args, rank, world, local):
    if rank != 0:
        return
    import __graft_entry__ as ge
    ib = ge.package()
    wl = make_workload(ib, args.workload)
    v, sec, cores = cpu_reference(ib, wl, args.steps, args.warmup)
    out = {
        "impl": "reference", "metric": baseline_metric(), "value": v, "unit": "cell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded PCG64 vorticity noise 1e-4 on the finest level",
        "config": bench_config(wl),
        "arm": {"precision": "fp64", "parallelism": "host threads"},
        "cpu_baseline": {"value": v, "unit": "cell-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} advance! steps of the full workload after {args.warmup} warm-up "
                                   "steps; FP64 NumPy/SciPy restatement of the reference (Julia is not installed); "
                                   "setup excluded"},
        "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="two_body_large")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the per-configuration summaries (2048^2 four cylinders, moving plate)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "mixed_tc"],
                    help="arithmetic of the timed arm (mixed: FP32 transforms + FP64 residual refinement)")
    ap.add_argument("--no-fp64-arm", action="store_true", help="skip timing the FP64 GPU path beside it")
    ap.add_argument("--refine-sweeps", type=int, default=0,
                    help="mixed precision: residual sweeps per solve (0: default policy, 1 or 2 everywhere)")
    ap.add_argument("--precision-table", action="store_true",
                    help="print the FP64 / FP32 / BF16x3 error table of the 2048^2 four-cylinder workload "
                         "at steps 100, 1000 and 2000 and exit")
    ap.add_argument("--learned-protocol", action="store_true",
                    help="print the learned warm start's moving-plate protocol (train on steps 0-2000 at f 0.2, "
                         "evaluate on 2000-4000 and on f 0.15 / 0.25) and a dt 0.001 stability probe, and exit")
    ap.add_argument("--next-rows", action="store_true",
                    help="print measurements of SchemeRKC, a translating grid, checkpoint files and batched "
                         "callbacks on the 1024^2 x 4 two-body workload, and exit")
    ap.add_argument("--profile-range", action="store_true",
                    help="bracket only the timed steps with cudaProfilerStart/Stop and skip the extras")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl != "reference" else args.warmup
    rank, world, local = dist_env()
    if args.learned_protocol:
        import __graft_entry__ as ge
        ib = ge.package()
        ge.build()
        ib.load_library()
        print(json.dumps({"learned_protocol": run_learned_protocol(ib),
                          "dt_probe": [run_dt_probe(ib, 0.001), run_dt_probe(ib, 0.0005)]}), flush=True)
        return
    if args.next_rows:
        import __graft_entry__ as ge
        ib = ge.package()
        ge.build()
        ib.load_library()
        print(json.dumps({"next_rows": run_next_rows(ib)}), flush=True)
        return
    if args.precision_table:
        import __graft_entry__ as ge
        ib = ge.package()
        ge.build()
        ib.load_library()
        print(json.dumps(run_precision_table(ib, make_workload(ib, "four_cylinders"))), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
