// Regularized delta weights (Reg / update!, src/streamfcn/structure-ops.jl:24-61, 114-171).
//
// This translation unit is compiled with -fmad=false: the reference evaluates the window
// coordinates h*(i-1+s) + x0 and r/h with separately rounded operations, and its 10-digit
// delta constants make the piecewise polynomial jump by ~1e-9 at r/h = 1, 2, 3.  A body point
// that sits on a grid line puts r/h within an ulp of such a breakpoint, so a fused multiply-add
// there can select the other branch; through the conditioning of the Schur matrix that would
// move the forces by ~1e-6.  Unfused arithmetic keeps every branch choice identical.
#include "ib_common.cuh"

namespace ib {

namespace {

// Yang-3 smooth delta times h (structure-ops.jl:114-171).  The constants are the reference's
// own (truncated to 10 digits there); they are kept, with the same evaluation order, because
// the forces depend on them directly.
__device__ double delta_h(double rf, double rb, double dr) {
  const double r = fabs(rf - rb);
  const double r1 = r / dr;
  const double r2 = r1 * r1;
  const double r3 = r2 * r1;
  const double r4 = r3 * r1;
  const double s3 = sqrt(3.0);
  if (r1 <= 1.0) {
    const double a5 = asin((1.0 / 2.0) * s3 * (2.0 * r1 - 1.0));
    const double a8 = sqrt(1.0 - 12.0 * r2 + 12.0 * r1);
    return 4.166666667e-2 * r4 + (-0.1388888889 + 3.472222222e-2 * a8) * r3 +
           (-7.121664902e-2 - 5.208333333e-2 * a8 + 0.2405626122 * a5) * r2 +
           (-0.2405626122 * a5 - 0.3792313933 + 0.1012731481 * a8) * r1 + 8.0187537413e-2 * a5 -
           4.195601852e-2 * a8 + 0.6485698427;
  } else if (r1 <= 2.0) {
    const double a6 = asin((1.0 / 2.0) * s3 * (-3.0 + 2.0 * r1));
    const double a9 = sqrt(-23.0 + 36.0 * r1 - 12.0 * r2);
    return -6.250000000e-2 * r4 + (0.4861111111 - 1.736111111e-2 * a9) * r3 +
           (-1.143175026 + 7.812500000e-2 * a9 - 0.1202813061 * a6) * r2 +
           (0.8751991178 + 0.3608439183 * a6 - 0.1548032407 * a9) * r1 - 0.2806563809 * a6 +
           8.22848104e-3 + 0.1150173611 * a9;
  } else if (r1 <= 3.0) {
    const double a1 = asin((1.0 / 2.0 * (2.0 * r1 - 5.0)) * s3);
    const double a7 = sqrt(-71.0 - 12.0 * r2 + 60.0 * r1);
    return 2.083333333e-2 * r4 + (3.472222222e-3 * a7 - 0.2638888889) * r3 +
           (1.214391675 - 2.604166667e-2 * a7 + 2.405626122e-2 * a1) * r2 +
           (-0.1202813061 * a1 - 2.449273192 + 7.262731481e-2 * a7) * r1 + 0.1523563211 * a1 +
           1.843201677 - 7.306134259e-2 * a7;
  }
  return 0.0;
}

// Reg update! (structure-ops.jl:37-61): one block per point.
__global__ void k_reg_update(Geometry g, const double* __restrict__ xb, int nb, int* __restrict__ body_idx,
                             double* __restrict__ weight, int* __restrict__ status) {
  __shared__ double d[4][kWin];
  __shared__ int idx[2];
  const int k = blockIdx.x;
  const double xk = xb[k], yk = xb[nb + k];
  const double h = g.h;
  if (threadIdx.x == 0) {
    bool ok = isfinite(xk) && isfinite(yk);
    int bi = 0, bj = 0;
    if (ok) {
      const double fx = floor((xk - g.x0) / h), fy = floor((yk - g.y0) / h);
      ok = fx > -1e9 && fx < 1e9 && fy > -1e9 && fy < 1e9;
      if (ok) { bi = (int)fx; bj = (int)fy; }
    }
    // 0-based window origin (bi - 7, bj - 7) must keep the 13x13 window inside both
    // flux grids: qx is (nx+1) x ny, qy is nx x (ny+1)
    if (!ok || bi - kSupp - 1 < 0 || bj - kSupp - 1 < 0 || bi - kSupp - 1 + kWin > g.nx ||
        bj - kSupp - 1 + kWin > g.ny) {
      atomicExch(status, 1);
      bi = kSupp + 1;
      bj = kSupp + 1;
    }
    idx[0] = bi;
    idx[1] = bj;
    body_idx[2 * k] = bi;
    body_idx[2 * k + 1] = bj;
  }
  __syncthreads();
  const int t = threadIdx.x;
  if (t < 4 * kWin) {
    const int which = t / kWin, s = t % kWin - kSupp;
    // x = h (bi - 1 + s) + x0 ; y = h (bj - 1 + s) + y0   (Julia 1-based face index)
    const double x = h * (double)(idx[0] - 1 + s) + g.x0;
    const double y = h * (double)(idx[1] - 1 + s) + g.y0;
    double v;
    if (which == 0) v = delta_h(x, xk, h);              // qx weights, x factor
    else if (which == 1) v = delta_h(y + h / 2, yk, h); // qx weights, y factor
    else if (which == 2) v = delta_h(x + h / 2, xk, h); // qy weights, x factor
    else v = delta_h(y, yk, h);                         // qy weights, y factor
    d[which][s + kSupp] = v;
  }
  __syncthreads();
  for (int e = t; e < 2 * kWin2; e += blockDim.x) {
    const int c = e / kWin2, r = e % kWin2;
    const int b = r / kWin, a = r % kWin;
    weight[(int64_t)k * 2 * kWin2 + e] = (c == 0) ? d[0][a] * d[1][b] : d[2][a] * d[3][b];
  }
}

}  // namespace

cudaError_t reg_update(const Geometry& g, const double* xb, int nb, int* body_idx, double* weight, int* status,
                       cudaStream_t s) {
  if (nb <= 0) return cudaSuccess;
  k_reg_update<<<nb, 64, 0, s>>>(g, xb, nb, body_idx, weight, status);
  return cudaGetLastError();
}

}  // namespace ib
