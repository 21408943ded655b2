/*
 * libibgb300 operator entry points: the stream-function operators of the reference's
 * StreamFcn module (exported at src/streamfcn/streamfcn.jl:17-22) on DEVICE pointers, run on
 * the handle's stream and synchronised before returning.  They use the same kernels as the
 * step and exist so each operator can be checked on its own (and called by a host that keeps
 * its arrays on the device).  Layouts are those of ibgb300.h; one level per call unless a
 * batch count is given (batched arrays are contiguous at their natural stride).
 */
#ifndef IBGB300_OPS_H
#define IBGB300_OPS_H

#include <stdint.h>

#include "ibgb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* FFTW plan_r2r(RODFT00, [1,2]) + mul! (src/streamfcn/fluid-ops.jl:25,49): unnormalised 2-D
 * DST-I of `batch` (nx-1)x(ny-1) arrays */
int ib_op_dst2(ib_handle* h, int32_t batch, const double* in, double* out);

/* The 1-D sine transform of the FFTW RODFT00 plan (fluid-ops.jl:24-25, one axis of it) as a
 * BF16x3 split-precision GEMM on the tensor cores: for each of `rows` FP32 lines of n-1 values
 * (n = nx for axis 0, ny for axis 1; a multiple of 128), out_k = sum_j in_j sin(pi j k / n),
 * k = 1..n-1 (half the RODFT00 value).  Relative error ~2^-16 of the row's magnitude; the
 * mixed-precision solves refine it away.  IB_ERR_UNSUPPORTED for other sizes. */
int ib_op_sine_lines_tc(ib_handle* h, int32_t axis, int32_t rows, const float* in, float* out);

/* LaplacianInv with lap_eigs (fluid-ops.jl:42-61): x = DST(DST(b) * scale / Λ) */
int ib_op_laplacian_inv(ib_handle* h, int32_t batch, const double* b, double* x);

/* Same result as ib_op_laplacian_inv, for callers that cannot allocate device memory while they
 * solve (their device memory belongs to another allocator or pool, or their loop cannot afford
 * an allocation's device-wide synchronisation).  No counterpart in the reference.  The work
 * buffer is a fixed 4,194,304-value FP64 array inside the library (32 MiB held on every device
 * that loads it), so batch * (nx-1)*(ny-1) must not exceed 4,194,304 (IB_ERR_INVALID
 * otherwise).  The first call on a device looks up the array's device address and should come
 * before any stream capture.  All calls share the array: calls that overlap on the GPU race. */
int ib_op_laplacian_inv_noalloc(ib_handle* h, int32_t batch, const double* b, double* x);

/* A[lev] and Ainv[lev] of A_Ainv_linearmaps (src/streamfcn/cnab/ops.jl:14-42); lev 1-based */
int ib_op_cn_a(ib_handle* h, int32_t lev, const double* b, double* x);
int ib_op_cn_ainv(ib_handle* h, int32_t lev, const double* b, double* x);

/* curl!(q, psi, psibc) multilevel (fluid-ops.jl:138-182); bc == NULL means a zero ring */
int ib_op_curl(ib_handle* h, const double* psi, const double* bc, double* q);

/* rot! = C^T (fluid-ops.jl:117-129) */
int ib_op_rot(ib_handle* h, const double* q, double* gamma);

/* coarsify!(gc, gf) (fluid-ops.jl:184-202), in place on gc */
int ib_op_coarsify(ib_handle* h, double* gc, const double* gf);

/* get_bc!(bc, r) (fluid-ops.jl:210-239) */
int ib_op_get_bc(ib_handle* h, const double* r, double* bc);

/* apply_bc!(r, bc, fac) (fluid-ops.jl:249-275), in place on r */
int ib_op_apply_bc(ib_handle* h, double* r, const double* bc, double fac);

/* Nonlinear (src/streamfcn/cnab/ops.jl:151-167) at level lev (1-based): avg_flux! of q + q0
 * with q0 = (u hc, v hc), direct_product! with ring bc, rot!, times 1/hc^2 */
int ib_op_nonlinear(ib_handle* h, int32_t lev, const double* q, double u, double v,
                    const double* gamma, const double* bc, double* nonlin);

/* Vort2Flux (fluid-ops.jl:438-472) on all levels: gamma is coarsened in place */
int ib_op_vort2flux(ib_handle* h, double* gamma, double* psi, double* q);

/* E = RegT (src/streamfcn/structure-ops.jl:88-105) on level-1 flux q (+ uniform q0 = (u, v)*h) */
int ib_op_reg_gather(ib_handle* h, const double* q, double u, double v, double* fb);

/* E^T = Reg (structure-ops.jl:63-86) */
int ib_op_reg_scatter(ib_handle* h, const double* fb, double* q);

/* HOST copies of the Schur matrix Bmat and its inverse (cnab/ops.jl:79-97), nf x nf
 * column-major, and of the delta data (structure-ops.jl:4-61): body_idx (nb x 2, the Julia
 * 1-based face index of each window centre) and weight [nb][2][13][13] (component, y, x). */
int ib_get_schur(ib_handle* h, double* bmat, double* binv);
int ib_get_reg(ib_handle* h, int32_t* body_idx, double* weight);

#ifdef __cplusplus
}
#endif

#endif /* IBGB300_OPS_H */
