/* libibgb300: ensembles of independent simulations stepped by one graph launch.
 *
 * No reference counterpart (the reference advances one problem per solve! call).  An ensemble
 * groups handles created by ib_create (any grid sizes, levels, bodies and precisions; same
 * device; same step count) and captures their advance! steps as parallel branches of one CUDA
 * graph, so that one launch advances every member by one step and their kernels share the GPU.
 * Each member's freestream value (and, for moving bodies, kinematics) enters through captured
 * host-to-device copies from pinned slots.  Moving members run their CG loop inside the graph
 * (a device-side convergence test), join after their first two steps (and first preconditioner
 * assembly) and keep their CG options while in the ensemble; the host reads their CG statistics
 * after every step and re-assembles preconditioners between launches.  The members' own state,
 * history and error reporting work as for single handles; a member must not be advanced on its
 * own while it belongs to an ensemble.  In an ensemble of two or more members, static mixed-
 * precision members are set to the level-by-level Vort2Flux (ib_set_vort2flux_order,
 * IB_V2F_SEQUENTIAL; it stays set afterwards): the members' branches fill the GPU between them,
 * and the all-levels order only adds work there (96 members on GB300: 14.0 vs 16.3 ms per step).
 */
#ifndef IBGB300_ENSEMBLE_H
#define IBGB300_ENSEMBLE_H

#include "ibgb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ib_ensemble ib_ensemble;

int ib_ensemble_create(ib_handle* const* members, int32_t n, ib_ensemble** out);
int ib_ensemble_destroy(ib_ensemble* e);

/* nsteps steps of every member: t[nsteps][n] (each member's time of the step; members may have
 * different time steps), uv[nsteps][n][2] (freestream per member and step); device_ms
 * (optional) receives the device time of the steps */
int ib_ensemble_advance_n(ib_ensemble* e, int32_t nsteps, const double* t, const double* uv, double* device_ms);

/* the same with moving members: kin[nsteps][6 per body of each moving member, in member
 * order] = r0x, r0y, v0x, v0y, theta, Omega (as ib_advance_kin) */
int ib_ensemble_advance_n_kin(ib_ensemble* e, int32_t nsteps, const double* t, const double* uv, const double* kin,
                              double* device_ms);

/* steps of every member per graph launch (1..8, default 1).  With k > 1 each launch carries k
 * consecutive steps of every member on the member's own branch, joined only at the end of the
 * launch: a member that finishes a step early (a moving member whose CG converged in few
 * iterations, a small grid) goes on with its next step instead of waiting for the slowest member.
 * The results are those of single-step launches, bit for bit.  Moving members' preconditioners
 * are re-assembled between launches only, and their CG statistics are read after each launch.
 * ib_ensemble_advance_n runs whole launches of k steps and the remaining steps one per launch. */
int ib_ensemble_set_steps_per_launch(ib_ensemble* e, int32_t k);

/* kernel launches per ensemble step (graph kernel nodes over all members) */
int ib_ensemble_info(ib_ensemble* e, int32_t* members, int32_t* kernels_per_step);

const char* ib_ensemble_last_error(const ib_ensemble* e);

#ifdef __cplusplus
}
#endif

#endif
