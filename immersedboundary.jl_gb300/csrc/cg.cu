// Moving bodies: rigid kinematics to body points, and the vector kernels of the Schur CG.
//
// Restates, with the corrections of the moving-body oracle, src/bodies/body-points.jl:47-76
// (update_bodies!: r = r0 + R(θ) xb, v = v0 + Ω R'(θ) xb) and the conjugate-gradient solve of
// src/streamfcn/cnab/ops.jl:104-114 (cg!(f, B, g) of IterativeSolvers 0.9.2, unpreconditioned).
// Every reduction has a fixed order (one block, fixed tree), so iterates are identical from run
// to run.
#include "ib_common.cuh"

namespace ib {

namespace {

// kin[b*6 + {0..5}] = r0x, r0y, v0x, v0y, theta, omega of body b
__global__ void k_body_points(const double* __restrict__ xb_body, const double* __restrict__ kin,
                              const int* __restrict__ body_of, int nb, double* __restrict__ xb,
                              double* __restrict__ vb) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += gridDim.x * blockDim.x) {
    const double* q = kin + 6 * body_of[k];
    const double c = cos(q[4]), s = sin(q[4]);
    const double bx = xb_body[k], by = xb_body[nb + k];
    xb[k] = q[0] + (c * bx - s * by);
    xb[nb + k] = q[1] + (s * bx + c * by);
    vb[k] = q[2] + q[5] * (-s * bx - c * by);
    vb[nb + k] = q[3] + q[5] * (c * bx - s * by);
  }
}

// y -= scale * v  (used for E(qs + q0) - ub h)
__global__ void k_axpy(double* __restrict__ y, const double* __restrict__ v, double a, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] += a * v[i];
}

constexpr int kRedThreads = 1024;

// out[0] = dot(a, b) with a fixed reduction order (one block)
__global__ void __launch_bounds__(kRedThreads) k_dot(const double* __restrict__ a, const double* __restrict__ b, int n,
                                                     double* __restrict__ out) {
  __shared__ double sm[kRedThreads / 32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += kRedThreads) acc = fma(a[i], b[i], acc);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = sm[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) out[0] = v;
  }
}

// CG scalars live in device memory: s[0] = rr, s[1] = p.Ap, s[2] = rr_new
// x += alpha p ; r -= alpha Ap   with alpha = rr / pAp
__global__ void k_cg_update_xr(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                               const double* __restrict__ Ap, const double* __restrict__ s, int n) {
  const double alpha = s[0] / s[1];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    r[i] = fma(-alpha, Ap[i], r[i]);
  }
}

// p = r + (rr_new / rr) p ; then rr = rr_new
__global__ void k_cg_update_p(double* __restrict__ p, const double* __restrict__ r, double* __restrict__ s, int n) {
  const double beta = s[2] / s[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = fma(beta, p[i], r[i]);
}

__global__ void k_cg_roll(double* s) {
  if (threadIdx.x == 0) s[0] = s[2];
}

inline int blocks(int n) { return (n + 255) / 256 < 1 ? 1 : (n + 255) / 256; }

// Device-side control of the CG loop in a captured step (a while-conditional graph node).
// sc: [0] r.z, [1] p.Ap, [2] new r.z, [3] rhs.rhs, [4] r.r, [5] target, [6] |rhs|;
// ctl: [0] iterations (as double), out: [0] iterations, [1] final and [2] initial relative
// residual, [3] 1 when the cap was reached
__global__ void k_cg_start(double* __restrict__ sc, double* __restrict__ ctl, double tol, int* __restrict__ status,
                           double* __restrict__ out, cudaGraphConditionalHandle cond) {
  if (threadIdx.x != 0) return;
  const double bn = sqrt(sc[3]), rn = sqrt(sc[4]);
  sc[5] = tol * bn;
  sc[6] = bn;
  ctl[0] = 0.0;
  out[2] = bn > 0.0 ? rn / bn : rn;
  const bool finite = isfinite(rn);
  if (!finite) status[1] = 1;
  cudaGraphSetConditional(cond, (finite && rn > sc[5]) ? 1u : 0u);
}

__global__ void k_cg_check(const double* __restrict__ sc, double* __restrict__ ctl, int maxiter, int* __restrict__ status,
                           cudaGraphConditionalHandle cond) {
  if (threadIdx.x != 0) return;
  ctl[0] += 1.0;
  const double rn = sqrt(sc[4]);
  const bool finite = isfinite(rn);
  if (!finite) status[1] = 1;
  cudaGraphSetConditional(cond, (finite && rn > sc[5] && ctl[0] < (double)maxiter) ? 1u : 0u);
}

__global__ void k_cg_finish(const double* __restrict__ sc, const double* __restrict__ ctl, double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  const double rn = sqrt(sc[4]), bn = sc[6];
  out[0] = ctl[0];
  out[1] = bn > 0.0 ? rn / bn : rn;
  out[3] = (isfinite(rn) && rn > sc[5]) ? 1.0 : 0.0;
}

}  // namespace

cudaError_t cg_start(double* sc, double* ctl, double tol, int* status, double* out, cudaGraphConditionalHandle cond,
                     cudaStream_t s) {
  k_cg_start<<<1, 32, 0, s>>>(sc, ctl, tol, status, out, cond);
  return cudaGetLastError();
}

cudaError_t cg_check(const double* sc, double* ctl, int maxiter, int* status, cudaGraphConditionalHandle cond,
                     cudaStream_t s) {
  k_cg_check<<<1, 32, 0, s>>>(sc, ctl, maxiter, status, cond);
  return cudaGetLastError();
}

cudaError_t cg_finish(const double* sc, const double* ctl, double* out, cudaStream_t s) {
  k_cg_finish<<<1, 32, 0, s>>>(sc, ctl, out);
  return cudaGetLastError();
}

cudaError_t body_points(const double* xb_body, const double* kin, const int* body_of, int nb, double* xb, double* vb,
                        cudaStream_t s) {
  if (nb <= 0) return cudaSuccess;
  k_body_points<<<blocks(nb), 256, 0, s>>>(xb_body, kin, body_of, nb, xb, vb);
  return cudaGetLastError();
}

cudaError_t vec_axpy(double* y, const double* v, double a, int n, cudaStream_t s) {
  k_axpy<<<blocks(n), 256, 0, s>>>(y, v, a, n);
  return cudaGetLastError();
}

cudaError_t vec_dot(const double* a, const double* b, int n, double* out, cudaStream_t s) {
  k_dot<<<1, kRedThreads, 0, s>>>(a, b, n, out);
  return cudaGetLastError();
}

cudaError_t cg_update_xr(double* x, double* r, const double* p, const double* Ap, const double* sc, int n,
                         cudaStream_t s) {
  k_cg_update_xr<<<blocks(n), 256, 0, s>>>(x, r, p, Ap, sc, n);
  return cudaGetLastError();
}

cudaError_t cg_update_p(double* p, const double* r, double* sc, int n, cudaStream_t s) {
  k_cg_update_p<<<blocks(n), 256, 0, s>>>(p, r, sc, n);
  k_cg_roll<<<1, 32, 0, s>>>(sc);
  return cudaGetLastError();
}

}  // namespace ib
