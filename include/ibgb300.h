/*
 * libibgb300 -- C ABI of the GB300-native immersed-boundary projection (IBPM / CNAB) step.
 *
 * Drop-in boundary for the stream-function / CNAB path of ImmersedBoundary.jl.  In the
 * reference the "plugin" is Julia dispatch: statetype(prob) / solvertype(prob) choose
 * CNAB.State / CNAB.Solver and solve! calls advance!(state, solver, t) once per step.  Each
 * entry point below names the reference function (file:line, relative to the
 * ImmersedBoundary.jl project root) that it replaces; the package's julia/IBGB300.jl holds
 * the Julia ccall binding.
 *
 * Conventions
 *   - every call returns an int status (IB_OK == 0); ib_last_error() gives the message;
 *   - host arrays are caller-owned FP64 in the reference's column-major layouts:
 *       gamma, psi, nonlin : (nx-1)*(ny-1) x nlevels  (Matrix nGamma x nlevel)
 *       q                  : nq x nlevels, each level [qx (nx+1)*ny ; qy nx*(ny+1)]
 *       fb                 : 2*nb, [fx_1..fx_nb, fy_1..fy_nb]
 *       xb                 : nb x 2 column-major, i.e. [x_1..x_nb, y_1..y_nb]
 *   - the library owns all device memory; nothing crosses the boundary per step except t,
 *     the freestream (u, v) at t and a status;
 *   - one handle owns one CUDA stream and its captured step graphs; a handle is not
 *     thread-safe, separate handles are independent.
 */
#ifndef IBGB300_H
#define IBGB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define IB_OK 0
#define IB_ERR_INVALID 1            /* bad argument / unsupported grid size */
#define IB_ERR_CUDA 2               /* CUDA runtime failure (message in ib_last_error) */
#define IB_ERR_NONFINITE 3          /* error("infinite flux"), src/streamfcn/structure-ops.jl:79-82 */
#define IB_ERR_BODY_OUT_OF_GRID 4   /* body point within 7 cells of the finest-grid edge */
#define IB_ERR_SINGULAR 5           /* zero / non-finite pivot while inverting the Schur matrix */
#define IB_ERR_CG_MAXITER 6         /* Schur CG hit its iteration cap */
#define IB_ERR_UNSUPPORTED 7        /* feature not supported for this handle or configuration */
#define IB_ERR_TIMEOUT 8            /* a device-side pipeline wait ran out (the kernel gave up and
                                       returned; the context stays usable) */

/* arithmetic of the fluid solve (state, nonlinear term, Schur solve and forces are FP64 in
 * every mode) */
#define IB_PREC_FP64 0   /* every sine transform in FP64 (the reference's arithmetic) */
#define IB_PREC_MIXED 1  /* FP32 sine transforms refined with float-float residuals (refine_sweeps);
                            state and stencils in float-float (two-float) arithmetic */
#define IB_PREC_MIXED_TC 2  /* as IB_PREC_MIXED, with every sine transform a BF16x3 split-precision
                               GEMM against the sine matrix on the tensor cores (FP32 accumulation);
                               both axes a multiple of 128 cells; Vort2Flux level by level */

/* time-stepping scheme (ib_problem.scheme) */
#define IB_SCHEME_CNAB 0  /* SchemeCNAB(dt), src/schemes.jl:19-26: the default */
#define IB_SCHEME_RKC 1   /* SchemeRKC(dt), src/schemes.jl:3-12: declared by the reference but given no
                             solver there; here the s-stage second-order Runge-Kutta-Chebyshev method
                             (damping 2/13) on dGamma/dt = nu lap(Gamma) + N(Gamma), explicit, then the
                             immersed-boundary projection with B' = E C Lap^-1 C^T E^T; FP64, bodies
                             fixed in the grid */

/* body motion */
#define IB_MOTION_STATIC 0          /* RigidBody{GridFrame}: E and B inverse built once */
#define IB_MOTION_PRESCRIBED 1      /* RigidBody{RelativeFrame}: xb in the body frame, rigid
                                       kinematics per step, E rebuilt and Fb solved by CG */

/* warm start of the moving-body Schur CG */
#define IB_WARM_PREVIOUS 0          /* previous step's Fb (cg! on qty.Fb, cnab/ops.jl:110) */
#define IB_WARM_EXTRAPOLATE 1       /* 2 Fb(n-1) - Fb(n-2) */
#define IB_WARM_ZERO 2              /* Fb = 0 (cold start, for comparisons) */
#define IB_WARM_LEARNED 3           /* learned prediction (include/ibgb300_learn.h); extrapolation
                                       until a network is trained */

typedef struct ib_problem {
  /* MultiLevel(UniformGrid(h, (x0, x1), (y0, y1)), nlevels), src/fluids/fluids.jl:53-95 */
  int32_t nx, ny, nlevels;
  double x0, y0, h;
  /* SchemeCNAB(dt), src/schemes.jl:19-26; beta = (1.5, -0.5) */
  double dt;
  double beta0, beta1;
  /* StreamFcnFluid(domain, freestream, Re), src/streamfcn/fluids.jl:49-58 */
  double re;
  /* BodyGroup(RigidBody(frame, xb, ds)...), src/bodies/bodies.jl:11-21, rigid-bodies.jl:4-10 */
  int32_t nbodies;
  const int32_t* body_npoints;  /* [nbodies] */
  const double* xb;             /* [2*nb] stacked points, column-major nb x 2 */
  const double* ds;             /* [nb] segment lengths */
  int32_t motion;               /* IB_MOTION_* */
  int32_t precision;            /* IB_PREC_* */
  int32_t device;               /* CUDA device ordinal */
  int32_t history_capacity;     /* steps of C_D / C_L kept on the device (0 -> 4096) */
  int32_t refine_sweeps;        /* IB_PREC_MIXED: residual sweeps per solve: 1 or 2 everywhere, or
                                   0 (default): 2, except 1 for the Vort2Flux solves of the third
                                   and coarser levels (they only feed boundary rings) */
  int32_t scheme;               /* IB_SCHEME_* (0: CNAB) */
  int32_t rkc_stages;           /* IB_SCHEME_RKC: stages s >= 2, or 0: the fewest whose stability
                                   interval covers 1.5 x dt x the finest level's viscous spectral
                                   radius 8 / (Re h^2) */
} ib_problem;

typedef struct ib_handle ib_handle;

/* initsolver(prob, state) -> CNAB.Solver(prob, state): src/streamfcn/cnab/timestepping.jl:193-249,
 * plus the zeroed CNAB.State buffers of initstate, src/streamfcn/cnab/states.jl:8-16.
 * Builds the transform tables, the delta weights (structure-ops.jl:24-61), assembles
 * Bmat column by column and inverts it (cnab/ops.jl:79-97), all on the device. */
int ib_create(const ib_problem* prob, ib_handle** out);

/* releases every device resource of the handle */
int ib_destroy(ib_handle* h);

/* copy!(state, src) of CNAB.State / StreamFcnQuantities (src/streamfcn/states.jl:90-100,
 * cnab/states.jl:1-16): upload Gamma, q, psi, the two nonlinear-history matrices
 * (nonlin1 = state.nonlin[1], nonlin2 = state.nonlin[2]), Fb and t.  NULL leaves a field. */
int ib_set_state(ib_handle* h, const double* gamma, const double* q, const double* psi,
                 const double* nonlin1, const double* nonlin2, const double* fb, double t);

/* read back state.qty.Γ, q, ψ, state.nonlin[1], state.nonlin[2], Fb and state.t; NULL skips */
int ib_get_state(ib_handle* h, double* gamma, double* q, double* psi, double* nonlin1,
                 double* nonlin2, double* fb, double* t);

/* Checkpoint files for restarts and for cross-checking with other implementations.  The
 * reference keeps snapshots in memory only (copy! of the state, src/streamfcn/states.jl:90-112,
 * cnab/states.jl:23-27; solve! resumes from a given state, src/solve.jl:188).  The file holds
 * what a restart needs: Gamma, q, psi, state.nonlin[1], state.nonlin[2], Fb, t, the step count
 * and, for moving bodies, the previous step's Fb; FP64 in the column-major layouts above after
 * a 56-byte header (magic "IBGB300C", int32 version 1, nx, ny, nlevels, npoints, moving flag,
 * two zeros, double t, int64 steps).  Loading checks that the handle's grid, levels, points and motion match.  An FP64
 * handle restarts to the same bits as an uninterrupted run; a mixed-precision one restarts its
 * solves' predictors from zero and agrees to the refinement tolerance. */
int ib_checkpoint_save(ib_handle* h, const char* path);
int ib_checkpoint_load(ib_handle* h, const char* path);

/* advance!(state, solver, t): src/streamfcn/cnab/timestepping.jl:253-290.  (u_inf, v_inf) is
 * fluid.freestream(t) (src/streamfcn/fluids.jl:82), evaluated by the caller; base_flux!
 * (src/streamfcn/fluid-ops.jl:403-417) runs on the device.  Synchronous: returns the step's
 * status (e.g. IB_ERR_NONFINITE for the reference's "infinite flux" error). */
int ib_advance(ib_handle* h, double t, double u_inf, double v_inf);

/* solver.vort2flux!(state.qty) (Vort2Flux, src/streamfcn/fluid-ops.jl:438-472) on the handle's
 * current state: coarsens Γ in place and recomputes ψ and q on every level. */
int ib_vort2flux(ib_handle* h);

/* The solve! time loop (src/solve.jl:198-212) for n steps without host callbacks:
 * advance! at t[i] with freestream (uv[2i], uv[2i+1]).  Replays the captured step graph;
 * synchronises once at the end and returns the first error. */
int ib_advance_n(ib_handle* h, int32_t n, const double* t, const double* uv);

/* advance! for moving bodies (RigidBody{RelativeFrame}; update_bodies!, src/bodies/body-points.jl:
 * 47-76, and the CG Binv of src/streamfcn/cnab/ops.jl:104-114, with the corrections the
 * reference's branch needs to run: the Ω field, point velocities, E rebuilt every step).
 * kin[6b..6b+5] = r0x, r0y, v0x, v0y, θ, Ω of body b at t (the frame's r, v, θ, Ω closures,
 * src/dynamics.jl:23-29, evaluated by the caller; bodies fixed in the grid pass zeros).
 * Fb solves B Fb = E(qs + q0) - ub h by conjugate gradients to ||r|| <= tol ||rhs||;
 * IB_ERR_CG_MAXITER if the cap is reached.  For static handles kin must be NULL. */
int ib_advance_kin(ib_handle* h, double t, double u_inf, double v_inf, const double* kin);

/* n moving-body steps: kin is [n][nbodies][6] */
int ib_advance_n_kin(ib_handle* h, int32_t n, const double* t, const double* uv, const double* kin);

/* CG options (the reference hard-codes maxiter=5000, cnab/ops.jl:110): tolerance on
 * ||r|| / ||rhs||, iteration cap and IB_WARM_* warm start.  Defaults 1e-10, 5000, PREVIOUS. */
int ib_set_cg_options(ib_handle* h, double tol, int32_t maxiter, int32_t warm_start);

/* Preconditioner of the moving-body CG (no reference counterpart; the reference runs plain cg!):
 * IB_PC_SCHUR_REF uses the inverse Schur matrix B_ref^-1 of a reference configuration (assembled
 * on the device like the static Binv of cnab/ops.jl:79-96: FP64, or FP32 transforms in a mixed-
 * precision handle, which P need not be exact for) as P in preconditioned CG.
 * It is assembled at the next step, then again every `refresh_steps` steps, or, with
 * refresh_steps = 0, once the CG iterations spent above those of the solve after the last
 * assembly have taken as long as that assembly (both timed on the host).  The stopping rule
 * ||r|| <= tol ||rhs|| is unchanged. */
#define IB_PC_NONE 0
#define IB_PC_SCHUR_REF 1
int ib_set_cg_preconditioner(ib_handle* h, int32_t mode, int32_t refresh_steps);

/* Order of the mixed-precision Vort2Flux (fluid-ops.jl:438-472 solves the levels coarse to fine,
 * each taking its boundary ring from the coarser solution).  IB_V2F_LEVELS finds every level's
 * ring first (harmonic ring transfer) and solves all levels in one batch; IB_V2F_SEQUENTIAL
 * keeps the reference's level order; IB_V2F_AUTO (the default) takes LEVELS up to 2^20 cells per
 * level where the grid has one-warp line passes.  The handle's step graphs are captured again;
 * a handle in an ensemble must not change it (the ensemble holds its own capture).  FP64
 * handles keep the reference order (accepted, no effect).  IB_ERR_UNSUPPORTED for LEVELS on a
 * grid without one-warp line passes. */
#define IB_V2F_AUTO 0
#define IB_V2F_LEVELS 1
#define IB_V2F_SEQUENTIAL 2
int ib_set_vort2flux_order(ib_handle* h, int32_t order);

/* number of preconditioner assemblies so far, the step of the last one (-1: none) and its
 * host-timed duration in seconds */
int ib_get_cg_preconditioner_stats(ib_handle* h, int32_t* assemblies, int64_t* last_step, double* last_seconds);

/* CG iterations and final relative residuals of the last `count` moving-body steps */
int ib_get_cg_stats(ib_handle* h, int32_t count, int32_t* iterations, double* residuals);

/* state.qty.points (BodyGroupPoints, src/bodies/body-points.jl:6-10): current positions and
 * velocities, stacked [x..., y...] */
int ib_get_body_points(ib_handle* h, double* xb, double* vb);

/* state.qty.stress of the last step (BodyStress, src/streamfcn/states.jl:3-7,53-84):
 * cd[b], cl[b] per body and, if fb_surface != NULL, the surface stress of every body as
 * consecutive column-major (n_b x 2) blocks. */
int ib_get_stress(ib_handle* h, double* cd, double* cl, double* fb_surface);

/* C_D / C_L of the last `count` steps (oldest first), per body: cd[s*nbodies + b].  This is
 * what a solve(...; save=(each_timestep(s -> s.qty.stress[b].CD),)) callback collects. */
int ib_get_force_history(ib_handle* h, int32_t count, double* cd, double* cl);

/* number of steps taken by this handle */
int64_t ib_step_count(const ib_handle* h);

/* block until every queued step of the handle has finished */
int ib_synchronize(ib_handle* h);

/* message of the last failed call on this handle (or of the last failed ib_create) */
const char* ib_last_error(const ib_handle* h);

/* static name of a status code */
const char* ib_status_string(int status);

#ifdef __cplusplus
}
#endif

#endif /* IBGB300_H */
