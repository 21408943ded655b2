// Multilevel Vort2Flux with all levels solved together (mixed precision, warp-per-line passes).
//
// Vort2Flux (src/streamfcn/fluid-ops.jl:438-472) solves the levels coarse to fine: level l's
// Poisson problem takes its boundary ring from psi_{l+1} (get_bc!, fluid-ops.jl:210-239), so the
// reference order is a chain of one-array solves.  Here the ring of every level is found first
// and all levels are then solved in one batch:
//
//   psi_{l+1} = psi0_{l+1} + H(ring_{l+1}),  psi0 = L^-1 Gamma (zero ring),  H = L^-1 apply_bc
//   ring_l    = get_bc(psi_{l+1})   (0.25 x values on the quarter lines of level l+1)
//
// The quarter lines lie n/4 cells inside level l+1.  Boundary mode k (sine along the side) of
// the harmonic part H decays across the grid as sinh(th_k (n-1-J)) / sinh(th_k n), 2 cosh th_k
// = 4 - 2 cos(pi (k+1)/n), i.e. by ~exp(-pi (k+1)/4) at the quarter lines: Kx (Ky) modes per
// side give H there to FP64 rounding.  ring_l is then a small FP64 product per level:
//   coef = St . sides(ring_{l+1}),  ring_l = ring(psi0_{l+1}) + Aring . coef.
// psi0 on the quarter lines comes from the first refinement sweeps: the previous call's psi
// plus an FP32 solve of its residual (x0) plus the next correction's spectrum evaluated on those
// lines (row sums in the y pass, column sums over the spectrum, then 1-D transforms).  The
// residual carries the rings of the previous call as a predictor, so psi0 above is psi with
// those rings and the chain carries only the change:
//   ring_l = get_bc(psi_old-ring_{l+1}) + Aring . coef(ring_{l+1} - ring_old_{l+1}).
#include <cmath>
#include <vector>

#include "dstw.cuh"

namespace ib {
namespace {

using wdst::kLB;
using wdst::kLines;
using wdst::line_dst;
using wdst::Shape;

// sin(pi m / 4) (row / column n/4) and sin(3 pi m / 4) (row / column 3n/4), m = (index+1) mod 8
__device__ __forceinline__ void quarter_weights(int m, float& qa, float& qb) {
  const float s = 0.70710678118654752f;
  const float mag = (m & 1) ? s : ((m & 3) == 2 ? 1.0f : 0.0f);
  qa = (m & 4) ? -mag : mag;
  qb = (m & 1) ? qa : -qa;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// line (b, k) of the transposed intermediate into U[1..nrow]
template <int NL>
__device__ __forceinline__ void load_line(float* U, const float* src, int nrow, int lane) {
  for (int J0 = lane; J0 < nrow; J0 += kLB * NL) {
    float v[kLB];
#pragma unroll
    for (int u = 0; u < kLB; ++u) v[u] = (J0 + NL * u < nrow) ? src[J0 + NL * u] : 0.0f;
#pragma unroll
    for (int u = 0; u < kLB; ++u)
      if (J0 + NL * u < nrow) U[J0 + NL * u + 1] = v[u];
  }
}

// y pass, spectrum only: S_y, multiply, store the spectrum in place, and the two quarter-row
// sums of its inverse, vrow[b][s][k] = sum_l sin(pi (l+1)(J_s+1)/ny) spec[k][l].
template <int P>
// 8 resident blocks per SM (64 registers), as the warp y pass the autotuner picks at the sizes
// that use the all-levels Vort2Flux
__global__ void __launch_bounds__(kLines * 32, 8)
k_wy_spec(Geometry g, DstAxis<float> ax, float* w, const float* m, int batch, float* vrow) {
  pdl_begin();
  using Sh = Shape<float, P, 32>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wi = threadIdx.x / 32, lane = threadIdx.x % 32;
  float* U = reinterpret_cast<float*>(smem_raw) + wi * Sh::kStride;
  float* D = U + Sh::kU;
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  float qa, qb;
  quarter_weights((lane + 1) & 7, qa, qb);  // l = lane + 32 u: (l+1) mod 8 is fixed per lane
  for (int col = blockIdx.x * kLines + wi; col < batch * ncol; col += gridDim.x * kLines) {
    const int b = col / ncol, k = col - b * ncol;
    float* line = w + (int64_t)b * g.nG + (int64_t)k * nrow;
    load_line<32>(U, line, nrow, lane);
    __syncwarp();
    line_dst<float, P, 32>(U, D, ax, lane, wi + 1);
    const float* mk = m + (int64_t)k * nrow;
    float sa = 0.0f, sb = 0.0f;
    for (int J0 = lane; J0 < nrow; J0 += kLB * 32) {
      float mv[kLB];
#pragma unroll
      for (int u = 0; u < kLB; ++u) mv[u] = (J0 + 32 * u < nrow) ? __ldg(&mk[J0 + 32 * u]) : 0.0f;
#pragma unroll
      for (int u = 0; u < kLB; ++u) {
        const int l = J0 + 32 * u;
        if (l < nrow) {
          const float v = U[l + 1] * mv[u];
          line[l] = v;
          sa = fmaf(qa, v, sa);
          sb = fmaf(qb, v, sb);
        }
      }
    }
    sa = warp_sum(sa);
    sb = warp_sum(sb);
    if (lane == 0) {
      vrow[(int64_t)(2 * b) * ncol + k] = sa;
      vrow[(int64_t)(2 * b + 1) * ncol + k] = sb;
    }
    __syncwarp();
  }
}

// y pass of the ring sweep: spec[k][l] + m[k][l] * (2-D transform of apply_bc(ring)), S_y, store.
// The transform of the ring's edge terms is separable:
//   sin(pi (l+1)/ny) (Fb_k + (-1)^l Ft_k) + sin(pi (k+1)/nx) (Fl_l + (-1)^k Fr_l)
// with Fb, Ft (Fl, Fr) the x (y) transforms of the bottom / top (left / right) ring sides.
template <int P>
__global__ void __launch_bounds__(kLines * 32, 8)
k_wy_ring(Geometry g, DstAxis<float> ax, float* w, const float* m, int batch, const float* sidex, const float* sidey,
          const float* sinx, const float* siny) {
  pdl_begin();
  using Sh = Shape<float, P, 32>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wi = threadIdx.x / 32, lane = threadIdx.x % 32;
  float* U = reinterpret_cast<float*>(smem_raw) + wi * Sh::kStride;
  float* D = U + Sh::kU;
  const int nx = g.nx, ny = g.ny, ncol = nx - 1, nrow = ny - 1;
  for (int col = blockIdx.x * kLines + wi; col < batch * ncol; col += gridDim.x * kLines) {
    const int b = col / ncol, k = col - b * ncol;
    float* line = w + (int64_t)b * g.nG + (int64_t)k * nrow;
    const float* mk = m + (int64_t)k * nrow;
    const float fb = sidex[(int64_t)(2 * b) * ncol + k], ft = sidex[(int64_t)(2 * b + 1) * ncol + k];
    const float sk = sinx[min(k + 1, nx - k - 1)];
    const float skr = (k & 1) ? -sk : sk;
    const float* fl = sidey + (int64_t)(2 * b) * nrow;
    const float* fr = sidey + (int64_t)(2 * b + 1) * nrow;
    // l = lane + 32 u: the parity of l is fixed per lane
    const float fbt = (lane & 1) ? fb - ft : fb + ft;
    for (int J0 = lane; J0 < nrow; J0 += kLB * 32) {
      float v[kLB], mv[kLB], a[kLB], c[kLB];
#pragma unroll
      for (int u = 0; u < kLB; ++u) {
        const int l = J0 + 32 * u;
        const bool ok = l < nrow;
        v[u] = ok ? line[l] : 0.0f;
        mv[u] = ok ? __ldg(&mk[l]) : 0.0f;
        a[u] = ok ? fl[l] : 0.0f;
        c[u] = ok ? fr[l] : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < kLB; ++u) {
        const int l = J0 + 32 * u;
        if (l < nrow) {
          const float sl = siny[min(l + 1, ny - l - 1)];
          const float bcs = fmaf(sl, fbt, sk * a[u] + skr * c[u]);
          U[l + 1] = fmaf(mv[u], bcs, v[u]);
        }
      }
    }
    __syncwarp();
    line_dst<float, P, 32>(U, D, ax, lane, wi + 1);
#pragma unroll 8
    for (int J = lane; J < nrow; J += 32) line[J] = U[J + 1];
    __syncwarp();
  }
}

// Column sums of the spectrum, in nchunk partial sums over k (chunks of 8 consecutive k, so
// the quarter weights are the same for every chunk):
//   ucolp[b][s][c][l] = sum_{k in chunk c} sin(pi (k+1)(I_s+1)/nx) spec[b][k][l]
constexpr int kColChunk = 32;  // k per thread
__global__ void k_colsum(Geometry g, const float* __restrict__ w, int batch, int nchunk, float* __restrict__ ucolp) {
  pdl_begin();
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y % nchunk, b = blockIdx.y / nchunk;
  if (l >= nrow || b >= batch) return;
  const int k0 = c * kColChunk;
  const float* src = w + (int64_t)b * g.nG + l;
  float sa = 0.0f, sb = 0.0f;
#pragma unroll
  for (int r = 0; r < kColChunk; r += 8) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = (k0 + r + u < ncol) ? src[(int64_t)(k0 + r + u) * nrow] : 0.0f;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      float qa, qb;
      quarter_weights((u + 1) & 7, qa, qb);  // k0 + r is a multiple of 8
      sa = fmaf(qa, v[u], sa);
      sb = fmaf(qb, v[u], sb);
    }
  }
  ucolp[((int64_t)(2 * b) * nchunk + c) * nrow + l] = sa;
  ucolp[((int64_t)(2 * b + 1) * nchunk + c) * nrow + l] = sb;
}

// ucol[t][l] = sum_c ucolp[t][c][l] in chunk order, t = 2 b + s
__global__ void k_colred(int nlines, int nchunk, int nrow, const float* __restrict__ ucolp, float* __restrict__ ucol) {
  pdl_begin();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nlines * nrow) return;
  const int t = (int)(i / nrow), l = (int)(i - (int64_t)t * nrow);
  const float* p = ucolp + (int64_t)t * nchunk * nrow + l;
  float s = 0.0f;
  for (int c0 = 0; c0 < nchunk; c0 += 8) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = (c0 + u < nchunk) ? p[(int64_t)(c0 + u) * nrow] : 0.0f;
#pragma unroll
    for (int u = 0; u < 8; ++u) s += v[u];
  }
  ucol[i] = s;
}

// 1-D DST-I (F convention) of `nlines` lines of ax.n-1 values, one warp per line; line t is
// (b = t / 2, s = t % 2), read at in + b in_b + s in_s and written to out + b out_b + s out_s
// (in place allowed).
template <int P>
__global__ void __launch_bounds__(kLines * 32)
k_lines(DstAxis<float> ax, const float* in, int64_t in_b, int64_t in_s, float* out, int64_t out_b, int64_t out_s,
        int nlines) {
  pdl_begin();
  using Sh = Shape<float, P, 32>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wi = threadIdx.x / 32, lane = threadIdx.x % 32;
  float* U = reinterpret_cast<float*>(smem_raw) + wi * Sh::kStride;
  float* D = U + Sh::kU;
  const int n1 = ax.n - 1;
  const int t = blockIdx.x * kLines + wi;
  if (t >= nlines) return;
  load_line<32>(U, in + (int64_t)(t >> 1) * in_b + (int64_t)(t & 1) * in_s, n1, lane);
  __syncwarp();
  line_dst<float, P, 32>(U, D, ax, lane, wi + 1);
  float* dst = out + (int64_t)(t >> 1) * out_b + (int64_t)(t & 1) * out_s;
  for (int j = lane; j < n1; j += 32) dst[j] = U[j + 1];
}

// ring_l from psi_{l+1} (with its previous ring) on the quarter lines, the previous psi + x0 +
// the next correction, plus (below the second-coarsest level) the harmonic part of the change of
// ring_{l+1}, Aring . coef_{l+1} (AringT: [nK][nbc], coalesced over the ring entries).  A block
// of kEvalWarps warps takes 32 ring nodes: warp w sums coefficients j = w, w + kEvalWarps, ...
// for all 32 (loads coalesced, five in flight), the partial sums are added in warp order in
// shared memory, and warp 0 finishes one node per lane.  FP64; ~nbc/32 blocks, so the FP64
// work spreads over the SMs (GB300 issues a warp's FP64 instruction over ~16 cycles).  `ring`
// holds the previous ring on entry and the new one on return; the change goes to dd (FP64, for
// the next coefficients), dring (float-float, for the residual) and the float sides.
constexpr int kEvalWarps = 8;
__global__ void __launch_bounds__(kEvalWarps * 32)
k_ring_eval(Geometry g, const int4* __restrict__ pts, const df64* __restrict__ xp, const float* __restrict__ x0,
            const float* __restrict__ qline, const double* __restrict__ AringT, const double* __restrict__ coef,
            int nK, double* __restrict__ dd, df64* __restrict__ dring, df64* __restrict__ ring,
            float* __restrict__ sidex, float* __restrict__ sidey) {
  pdl_begin();
  __shared__ double part[kEvalWarps][32];
  const int w = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int idx = blockIdx.x * 32 + lane;
  // warp 0 starts the node's own loads before its share of the sum
  double v = 0.0;
  df64 old(0.0f);
  if (w == 0 && idx < g.nbc) {
    const int4 p = pts[idx];
    old = ring[idx];
    v = (double)xp[p.x] + ((double)x0[p.x] + (double)qline[p.y]);
    if (p.z >= 0) v = 0.5 * (v + ((double)xp[p.z] + ((double)x0[p.z] + (double)qline[p.w])));
  }
  double h = 0.0;
  if (coef && idx < g.nbc) {
    const double* a = AringT + idx;
    constexpr int U = 5;
    int j = w;
    for (; j + (U - 1) * kEvalWarps < nK; j += U * kEvalWarps) {
      double av[U];
#pragma unroll
      for (int u = 0; u < U; ++u) av[u] = a[(int64_t)(j + u * kEvalWarps) * g.nbc];
#pragma unroll
      for (int u = 0; u < U; ++u) h = fma(av[u], __ldg(&coef[j + u * kEvalWarps]), h);
    }
    for (; j < nK; j += kEvalWarps) h = fma(a[(int64_t)j * g.nbc], __ldg(&coef[j]), h);
  }
  part[w][lane] = h;
  __syncthreads();
  if (w != 0 || idx >= g.nbc) return;
  h = 0.0;
#pragma unroll
  for (int k = 0; k < kEvalWarps; ++k) h += part[k][lane];
  v = 0.25 * v + h;
  const double d = v - (double)old;
  dd[idx] = d;
  dring[idx] = df64(d);
  ring[idx] = df64(v);
  const float df = (float)d;
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  if (idx > g.B && idx < g.B + g.nx) sidex[idx - g.B - 1] = df;
  else if (idx > g.T && idx < g.T + g.nx) sidex[ncol + idx - g.T - 1] = df;
  else if (idx > g.L && idx < g.L + g.ny) sidey[idx - g.L - 1] = df;
  else if (idx > g.R && idx < g.R + g.ny) sidey[nrow + idx - g.R - 1] = df;
}

// coef_l: the first Kx (Ky) sine coefficients of the bottom, top (left, right) ring sides,
// coef[j] = sum_i St[j][i] side_i (S convention, 2 sin).  One block of kCoefThreads per
// coefficient (nK blocks spread the FP64 work over the SMs), a strided sum per thread, then a
// fixed-order tree in shared memory; FP64.
constexpr int kCoefThreads = 256;
__global__ void __launch_bounds__(kCoefThreads)
k_ring_coef(Geometry g, const double* __restrict__ ringd, const double* __restrict__ St, int Kx, int Ky,
            double* __restrict__ coef) {
  pdl_begin();
  __shared__ double red[kCoefThreads];
  const int j = blockIdx.x, tid = threadIdx.x;
  const int nK = 2 * Kx + 2 * Ky;
  if (j >= nK) return;
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const double* row;
  const double* side;
  int len;
  if (j < 2 * Kx) {
    const int k = j < Kx ? j : j - Kx;
    row = St + (int64_t)k * ncol;
    side = ringd + (j < Kx ? g.B : g.T) + 1;
    len = ncol;
  } else {
    const int jj = j - 2 * Kx;
    const int k = jj < Ky ? jj : jj - Ky;
    row = St + (int64_t)Kx * ncol + (int64_t)k * nrow;
    side = ringd + (jj < Ky ? g.L : g.R) + 1;
    len = nrow;
  }
  double s = 0.0;
  for (int i = tid; i < len; i += kCoefThreads) s = fma(row[i], side[i], s);
  red[tid] = s;
  __syncthreads();
#pragma unroll
  for (int o = kCoefThreads / 2; o > 0; o >>= 1) {
    if (tid < o) red[tid] += red[tid + o];
    __syncthreads();
  }
  if (tid == 0) coef[j] = red[0];
}

template <int P>
size_t line_smem() {
  return (size_t)kLines * Shape<float, P, 32>::kStride * sizeof(float);
}

// harmonic decay g_k(J) = sinh(th (m-1-J)) / (2 n sinh(th m)), 2 cosh th = 4 - 2 cos(pi (k+1)/n),
// for J = 0..m-2, written stably with exponentials
void decay_table(int n, int m, int K, std::vector<double>& out) {
  const double pi = 3.14159265358979323846;
  out.assign((size_t)K * (m - 1), 0.0);
  for (int k = 0; k < K; ++k) {
    const double th = std::acosh(2.0 - std::cos(pi * (k + 1) / n));
    const double den = 1.0 - std::exp(-2.0 * th * m);
    for (int J = 0; J < m - 1; ++J) {
      const double num = std::exp(-th * (J + 1)) * (1.0 - std::exp(-2.0 * th * (m - 1 - J)));
      out[(size_t)k * (m - 1) + J] = num / den / (2.0 * n);
    }
  }
}

// modes kept for a side along an axis of n cells whose nearest quarter-line node is d cells
// away: the smallest K with 2 sum_{k >= K} exp(-th_k d) below 1e-17
int modes_kept(int n, int d) {
  const double pi = 3.14159265358979323846;
  std::vector<double> e(n - 1);
  for (int k = 0; k < n - 1; ++k) e[k] = std::exp(-std::acosh(2.0 - std::cos(pi * (k + 1) / n)) * d);
  double tail = 0.0;
  int K = n - 1;
  for (int k = n - 2; k >= 0; --k) {
    tail += 2.0 * e[k];
    if (tail >= 1e-17) break;
    K = k;
  }
  return K;
}

}  // namespace

#define CE_V(x)                      \
  do {                               \
    cudaError_t e_ = (x);            \
    if (e_ != cudaSuccess) return e_; \
  } while (0)

template <int P>
static cudaError_t launch_lines_p(const DstAxis<float>& ax, const float* in, int64_t in_b, int64_t in_s, float* out,
                                  int64_t out_b, int64_t out_s, int nlines, cudaStream_t s) {
  const size_t smem = line_smem<P>();
  cudaError_t e = set_smem_limit((const void*)k_lines<P>, smem);
  if (e != cudaSuccess) return e;
  CE_V(launch_k(k_lines<P>, dim3((nlines + kLines - 1) / kLines), dim3(kLines * 32), smem, s, ax, in, in_b, in_s, out, out_b, out_s, nlines));
  return cudaGetLastError();
}

// one-warp (wNL = 32) axes only
#define IB_V2F_P(X) X(1) X(2) X(3) X(4) X(6) X(8) X(12) X(16) X(24) X(32)

cudaError_t v2f_lines(const DstAxis<float>& ax, const float* in, int64_t in_b, int64_t in_s, float* out,
                      int64_t out_b, int64_t out_s, int nlines, cudaStream_t s) {
  if (nlines <= 0) return cudaSuccess;
  if (ax.wNL != 32) return cudaErrorInvalidValue;
  switch (ax.wP) {
#define IB_C(P) \
  case P: return launch_lines_p<P>(ax, in, in_b, in_s, out, out_b, out_s, nlines, s);
    IB_V2F_P(IB_C)
#undef IB_C
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t v2f_yspec(const Geometry& g, const DstAxis<float>& ax, float* w, const float* m, int batch, float* vrow,
                      cudaStream_t s) {
  if (ax.wNL != 32 || ax.n != g.ny) return cudaErrorInvalidValue;
  ProfScope prof(kClassYPass, s);
  const int blocks = (batch * (g.nx - 1) + kLines - 1) / kLines;
  switch (ax.wP) {
#define IB_C(P)                                                                          \
  case P: {                                                                              \
    const size_t smem = line_smem<P>();                                                  \
    cudaError_t e = set_smem_limit((const void*)k_wy_spec<P>, smem);                     \
    if (e != cudaSuccess) return e;                                                      \
    CE_V(launch_k(k_wy_spec<P>, dim3(blocks), dim3(kLines * 32), smem, s, g, ax, w, m, batch, vrow));            \
    return cudaGetLastError();                                                           \
  }
    IB_V2F_P(IB_C)
#undef IB_C
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t v2f_yring(const Geometry& g, const DstAxis<float>& axy, const DstAxis<float>& axx, float* w,
                      const float* m, int batch, const float* sidex, const float* sidey, cudaStream_t s) {
  if (axy.wNL != 32 || axy.n != g.ny || axx.n != g.nx) return cudaErrorInvalidValue;
  ProfScope prof(kClassYPass, s);
  const int blocks = (batch * (g.nx - 1) + kLines - 1) / kLines;
  switch (axy.wP) {
#define IB_C(P)                                                                                           \
  case P: {                                                                                               \
    const size_t smem = line_smem<P>();                                                                   \
    cudaError_t e = set_smem_limit((const void*)k_wy_ring<P>, smem);                                      \
    if (e != cudaSuccess) return e;                                                                       \
    CE_V(launch_k(k_wy_ring<P>, dim3(blocks), dim3(kLines * 32), smem, s, g, axy, w, m, batch, sidex, sidey, axx.sintab, axy.sintab)); \
    return cudaGetLastError();                                                                            \
  }
    IB_V2F_P(IB_C)
#undef IB_C
    default: return cudaErrorInvalidValue;
  }
}
#undef IB_V2F_P

cudaError_t v2f_colsum(const Geometry& g, const RingPlan& rp, const float* w, int batch, cudaStream_t s) {
  const int nrow = g.ny - 1;
  dim3 grid((nrow + 127) / 128, batch * rp.nchunk);
  CE_V(launch_k(k_colsum, grid, dim3(128), 0, s, g, w, batch, rp.nchunk, rp.ucolp));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int64_t n = (int64_t)2 * batch * nrow;
  CE_V(launch_k(k_colred, dim3((int)((n + 255) / 256)), dim3(256), 0, s, 2 * batch, rp.nchunk, nrow, rp.ucolp, rp.ucol));
  return cudaGetLastError();
}

cudaError_t v2f_ring_eval(const Geometry& g, const RingPlan& rp, int l, const df64* xp_up, const float* x0_up,
                          df64* ring_l, cudaStream_t s) {
  const int up = l + 1;
  const double* coef = (up < g.nlev - 1) ? rp.coef + (int64_t)up * rp.nK : nullptr;
  return launch_k(k_ring_eval, dim3((g.nbc + 31) / 32), dim3(kEvalWarps * 32), 0, s, g, (const int4*)rp.pts, xp_up,
                  x0_up, (const float*)(rp.qline + (int64_t)up * rp.qls), (const double*)rp.Aring, coef, rp.nK,
                  rp.ringd + (int64_t)l * g.nbc, reinterpret_cast<df64*>(rp.dring) + (int64_t)l * g.nbc, ring_l,
                  rp.sidex + (int64_t)l * 2 * (g.nx - 1), rp.sidey + (int64_t)l * 2 * (g.ny - 1));
}

cudaError_t v2f_ring_coef(const Geometry& g, const RingPlan& rp, int l, cudaStream_t s) {
  return launch_k(k_ring_coef, dim3(rp.nK), dim3(kCoefThreads), 0, s, g, (const double*)(rp.ringd + (int64_t)l * g.nbc),
                  (const double*)rp.St, rp.Kx, rp.Ky, rp.coef + (int64_t)l * rp.nK);
}

// Host tables: truncation, St, Aring and the quarter-line nodes of each ring entry.
cudaError_t RingPlan::build(const Geometry& g) {
  const int nx = g.nx, ny = g.ny, ncol = nx - 1, nrow = ny - 1, L = g.nlev;
  const int nx4 = nx / 4, ny4 = ny / 4;
  const double pi = 3.14159265358979323846;
  Kx = modes_kept(nx, ny4);  // bottom / top modes, nearest quarter-line node ny/4 cells away
  Ky = modes_kept(ny, nx4);
  nK = 2 * Kx + 2 * Ky;
  qls = 2 * (int64_t)ncol + 2 * (int64_t)nrow;
  nchunk = (ncol + kColChunk - 1) / kColChunk;
  std::vector<double> st((size_t)Kx * ncol + (size_t)Ky * nrow);
  for (int k = 0; k < Kx; ++k)
    for (int i = 0; i < ncol; ++i) st[(size_t)k * ncol + i] = 2.0 * std::sin(pi * (double)(k + 1) * (i + 1) / nx);
  for (int k = 0; k < Ky; ++k)
    for (int j = 0; j < nrow; ++j)
      st[(size_t)Kx * ncol + (size_t)k * nrow + j] = 2.0 * std::sin(pi * (double)(k + 1) * (j + 1) / ny);
  std::vector<double> gx, hy;
  decay_table(nx, ny, Kx, gx);  // [k][J]: bottom-side mode k at row J
  decay_table(ny, nx, Ky, hy);  // [l][I]: left-side mode l at column I
  auto stx = [&](int k, int I) { return st[(size_t)k * ncol + I]; };
  auto sty = [&](int k, int J) { return st[(size_t)Kx * ncol + (size_t)k * nrow + J]; };
  // harmonic response at node (J, I) per coefficient, accumulated with weight wt
  auto add_node = [&](double* a, int J, int I, double wt) {
    for (int k = 0; k < Kx; ++k) {
      a[k] += wt * stx(k, I) * gx[(size_t)k * nrow + J];
      a[Kx + k] += wt * stx(k, I) * gx[(size_t)k * nrow + (ny - 2 - J)];
    }
    for (int k = 0; k < Ky; ++k) {
      a[2 * Kx + k] += wt * sty(k, J) * hy[(size_t)k * ncol + I];
      a[2 * Kx + Ky + k] += wt * sty(k, J) * hy[(size_t)k * ncol + (nx - 2 - I)];
    }
  };
  std::vector<double> A((size_t)g.nbc * nK, 0.0);
  std::vector<int4> P(g.nbc);
  for (int idx = 0; idx < g.nbc; ++idx) {
    // the nodes get_bc! reads (fluid-ops.jl:210-239): column nx/4-1 or 3nx/4-1 (left / right
    // blocks) or row ny/4-1 or 3ny/4-1 (bottom / top), averaged pairs at odd ring entries
    int J1, I1, J2 = -1, I2 = -1, q1, q2 = -1;
    if (idx < g.B) {
      const bool right = idx >= g.R;
      const int jb = idx - (right ? g.R : g.L);
      const int I = right ? 3 * nx4 - 1 : nx4 - 1;
      const int qb = 2 * ncol + (right ? nrow : 0);
      const int t = (jb + 1) >> 1;
      J1 = ny4 - 1 + ((jb & 1) ? t : jb >> 1);
      I1 = I;
      q1 = qb + J1;
      if (jb & 1) { J2 = ny4 - 2 + t; I2 = I; q2 = qb + J2; }
    } else {
      const bool top = idx >= g.T;
      const int ib = idx - (top ? g.T : g.B);
      const int J = top ? 3 * ny4 - 1 : ny4 - 1;
      const int qb = top ? ncol : 0;
      const int t = (ib + 1) >> 1;
      J1 = J;
      I1 = nx4 - 1 + ((ib & 1) ? t : ib >> 1);
      q1 = qb + I1;
      if (ib & 1) { J2 = J; I2 = nx4 - 2 + t; q2 = qb + I2; }
    }
    double* a = A.data() + (size_t)idx * nK;
    if (J2 < 0) {
      add_node(a, J1, I1, 0.25);
      P[idx] = make_int4(J1 * ncol + I1, q1, -1, -1);
    } else {
      add_node(a, J1, I1, 0.125);
      add_node(a, J2, I2, 0.125);
      P[idx] = make_int4(J1 * ncol + I1, q1, J2 * ncol + I2, q2);
    }
  }
  auto up = [&](auto*& dst, const auto& src) -> cudaError_t {
    const size_t bytes = src.size() * sizeof(src[0]);
    cudaError_t e = cudaMalloc(&dst, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(dst, src.data(), bytes, cudaMemcpyHostToDevice);
    return e;
  };
  cudaError_t e;
  if ((e = up(St, st)) != cudaSuccess) return e;
  std::vector<double> AT((size_t)nK * g.nbc);  // [nK][nbc]: the evaluation kernel reads it by node
  for (int idx = 0; idx < g.nbc; ++idx)
    for (int j = 0; j < nK; ++j) AT[(size_t)j * g.nbc + idx] = A[(size_t)idx * nK + j];
  if ((e = up(Aring, AT)) != cudaSuccess) return e;
  if ((e = up(pts, P)) != cudaSuccess) return e;
  auto zero = [&](auto*& dst, int64_t n) -> cudaError_t {
    cudaError_t e2 = cudaMalloc(&dst, sizeof(*dst) * n);
    if (e2 == cudaSuccess) e2 = cudaMemset(dst, 0, sizeof(*dst) * n);
    return e2;
  };
  if ((e = zero(vrow, (int64_t)L * 2 * ncol)) != cudaSuccess) return e;
  if ((e = zero(ucolp, (int64_t)L * 2 * nchunk * nrow)) != cudaSuccess) return e;
  if ((e = zero(ucol, (int64_t)L * 2 * nrow)) != cudaSuccess) return e;
  if ((e = zero(dring, (int64_t)L * g.nbc)) != cudaSuccess) return e;
  if ((e = zero(qline, (int64_t)L * qls)) != cudaSuccess) return e;
  if ((e = zero(sidex, (int64_t)L * 2 * ncol)) != cudaSuccess) return e;
  if ((e = zero(sidey, (int64_t)L * 2 * nrow)) != cudaSuccess) return e;
  if ((e = zero(ringd, (int64_t)L * g.nbc)) != cudaSuccess) return e;
  if ((e = zero(coef, (int64_t)L * nK)) != cudaSuccess) return e;
  return cudaSuccess;
}

void RingPlan::release() {
  for (void* p : {(void*)St, (void*)Aring, (void*)pts, (void*)vrow, (void*)ucolp, (void*)ucol, (void*)qline,
                  (void*)sidex, (void*)sidey, (void*)ringd, (void*)dring, (void*)coef})
    if (p) cudaFree(p);
  St = nullptr; Aring = nullptr; pts = nullptr; vrow = nullptr; ucolp = nullptr; ucol = nullptr; qline = nullptr;
  sidex = nullptr; sidey = nullptr; ringd = nullptr; dring = nullptr; coef = nullptr;
}

}  // namespace ib
