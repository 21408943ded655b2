/* libibgb300: learned warm start of the moving-body Schur CG.
 *
 * No reference counterpart: the reference solves B Fb = rhs with cg! started from the previous
 * Fb (src/streamfcn/cnab/ops.jl:104-114).  Here a small perceptron reads the step's body
 * kinematics and the last two force vectors and predicts F_n as the CG starting point
 * (IB_WARM_LEARNED in ib_set_cg_options); CG then runs to the same tolerance, so the learned
 * part changes the iteration count only.  The network is trained on the device, by this
 * library's own kernels, on (features, F_n) samples recorded while stepping.
 *
 *   features x = [r0x, r0y, v0x, v0y, theta, Omega per body (the kin rows of ib_advance_kin),
 *                 F_{n-1}, F_{n-2}]                         (6 nbodies + 2 nf values)
 *   target   y = F_n - (2 F_{n-1} - F_{n-2})               (nf values)
 *   network  hidden tanh layers of equal width, linear output; inputs and targets normalised
 *            per component by the recorded samples' mean and standard deviation
 *   weights  BF16 for the products (FP32 accumulation), FP32 master copies updated by Adam
 *   start    F_n ~ 2 F_{n-1} - F_{n-2} + blend * correction, blend validated on held-out samples
 * Parameters are stored layer by layer: W_l (dims[l+1] x dims[l], row-major), then b_l.
 */
#ifndef IBGB300_LEARN_H
#define IBGB300_LEARN_H

#include "ibgb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* create the network for a moving-body handle (IB_MOTION_PRESCRIBED): `hidden_layers` layers
 * of width `hidden`, a ring of `capacity` samples, seeded Xavier-uniform weights (the output
 * layer starts at zero, i.e. at plain extrapolation) */
int ib_learn_init(ib_handle* h, int32_t hidden, int32_t hidden_layers, int32_t capacity, uint64_t seed);

/* record (features, F_n) after every moving-body step from now on (on = 1) or stop (0) */
int ib_learn_collect(ib_handle* h, int32_t on);

/* number of recorded samples (at most the capacity) */
int ib_learn_sample_count(ib_handle* h, int32_t* count);

/* minibatch Adam on the recorded samples (normalisation taken from them); `final_loss` is the
 * mean squared normalised error over the last epoch */
int ib_learn_train(ib_handle* h, int32_t epochs, int32_t batch, double lr, uint64_t seed, double* final_loss);

/* held-out check of the last training (the most recent tenth of the samples, not trained on):
 * `blend` in [0, 1] is the weight given to the network's correction, the least-squares optimum
 * on the held-out rows (at most the 256 most recent) in the norm the CG start residual is
 * measured in, |B (blend q - t)| with B the Schur operator of the configuration at training
 * (0 means plain extrapolation); `rel_err` the held-out squared error of the blended start in
 * that norm relative to plain extrapolation's (-1 when there were too few samples) */
int ib_learn_validation(ib_handle* h, double* blend, double* rel_err);

/* layer widths (nlayers + 1 values: features, hidden..., forces) */
int ib_learn_layout(ib_handle* h, int32_t* nlayers, int32_t* dims, int32_t max_dims);
int ib_learn_param_count(ib_handle* h, int64_t* nparam);
int ib_learn_get_params(ib_handle* h, float* params);
int ib_learn_set_params(ib_handle* h, const float* params);

/* weight of the network's correction in the warm start, in [0, 1] (0: plain extrapolation);
 * replaces the validated value until the next training */
int ib_learn_set_blend(ib_handle* h, double blend);

/* a trained network with its normalisation, to reuse it on another handle of the same layout
 * (another frequency, say): n = nparam + 2 dims[0] + 2 dims[last] + 1 floats: the parameters,
 * mu_x, sd_x, mu_y, sd_y, then the blend.  Import marks the network trained. */
int ib_learn_export(ib_handle* h, float* buf, int64_t n);
int ib_learn_import(ib_handle* h, const float* buf, int64_t n);

/* loss and parameter gradients of the network (normalisation not applied) on `rows` host rows
 * of inputs x [rows][dims[0]] and targets y [rows][dims[last]]: the training kernels, exposed
 * for gradient checks */
int ib_learn_gradients(ib_handle* h, int32_t rows, const float* x, const float* y, float* grad, double* loss);

/* initial relative residuals ||rhs - B x0|| / ||rhs|| of the last `count` CG solves */
int ib_get_cg_start_residuals(ib_handle* h, int32_t count, double* r0);

#ifdef __cplusplus
}
#endif

#endif
