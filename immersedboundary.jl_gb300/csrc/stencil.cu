// Stencil kernels of the stream-function discretisation.
//
// Each kernel restates one operator of src/streamfcn/fluid-ops.jl (cited per kernel) on the
// reference's own column-major layouts.  Grid-stride loops, one thread per output value.
#include "ib_common.cuh"

namespace ib {

namespace {

constexpr int kThreads = 256;

inline int blocks_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b > 65535LL * 8) b = 65535LL * 8;
  return (int)(b < 1 ? 1 : b);
}

// x * s for a power of two s: exact, so a float-float value scales part by part (the general
// float-float product would spend ~7 FP32 operations on it)
template <typename T>
__device__ __forceinline__ T xscale(T x, float s) {
  return x * T(s);
}
template <>
__device__ __forceinline__ df64 xscale<df64>(df64 x, float s) {
  return df64(x.hi * s, x.lo * s);
}

// get_bc! value at ring index idx (fluid-ops.jl:210-239), including the final *0.25.
template <typename T>
__device__ __forceinline__ T ring_value(const Geometry& g, const T* __restrict__ r, int idx) {
  const int nx = g.nx, ny = g.ny, ncol = nx - 1;
  const int nx4 = nx / 4, ny4 = ny / 4;
  T v;
  if (idx < g.B) {  // left (idx < R) or right block, node along y
    const bool right = idx >= g.R;
    const int jb = idx - (right ? g.R : g.L);
    const int col = right ? 3 * nx4 - 1 : nx4 - 1;
    if ((jb & 1) == 0) {
      const int t = jb >> 1;
      v = r[(ny4 - 1 + t) * ncol + col];
    } else {
      const int t = (jb + 1) >> 1;
      v = xscale(r[(ny4 - 1 + t) * ncol + col] + r[(ny4 - 2 + t) * ncol + col], 0.5f);
    }
  } else {  // bottom (idx < T) or top block, node along x
    const bool top = idx >= g.T;
    const int ib = idx - (top ? g.T : g.B);
    const int row = top ? 3 * ny4 - 1 : ny4 - 1;
    if ((ib & 1) == 0) {
      const int t = ib >> 1;
      v = r[row * ncol + nx4 - 1 + t];
    } else {
      const int t = (ib + 1) >> 1;
      v = xscale(r[row * ncol + nx4 - 1 + t] + r[row * ncol + nx4 - 2 + t], 0.5f);
    }
  }
  return xscale(v, 0.25f);
}

template <typename T>
__global__ void k_get_bc(Geometry g, const T* __restrict__ r, T* __restrict__ bc, int batch, T extra) {
  pdl_begin();
  const int64_t total = (int64_t)batch * g.nbc;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(t / g.nbc), idx = (int)(t - (int64_t)b * g.nbc);
    bc[t] = ring_value(g, r + (int64_t)b * g.nG, idx) * extra;
  }
}

// apply_bc! (fluid-ops.jl:249-275): rows first, then columns (same order as the reference).
template <typename T>
__global__ void k_apply_bc_rows(Geometry g, T* __restrict__ r, const T* __restrict__ bc, T fac, int batch) {
  pdl_begin();
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const int64_t total = (int64_t)batch * ncol;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(t / ncol), I = (int)(t - (int64_t)b * ncol);
    T* rr = r + (int64_t)b * g.nG;
    const T* bb = bc + (int64_t)b * g.nbc;
    rr[I] += fac * bb[g.B + 1 + I];
    rr[(nrow - 1) * ncol + I] += fac * bb[g.T + 1 + I];
  }
}
template <typename T>
__global__ void k_apply_bc_cols(Geometry g, T* __restrict__ r, const T* __restrict__ bc, T fac, int batch) {
  pdl_begin();
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const int64_t total = (int64_t)batch * nrow;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(t / nrow), J = (int)(t - (int64_t)b * nrow);
    T* rr = r + (int64_t)b * g.nG;
    const T* bb = bc + (int64_t)b * g.nbc;
    rr[J * ncol] += fac * bb[g.L + 1 + J];
    rr[J * ncol + ncol - 1] += fac * bb[g.R + 1 + J];
  }
}

// coarsify! (fluid-ops.jl:184-202)
template <typename T>
__global__ void k_coarsify(Geometry g, T* __restrict__ gc, const T* __restrict__ gf, int batch, int64_t stride) {
  pdl_begin();
  const int ncol = g.nx - 1;
  const int ct = g.nx / 2 - 1, cs = g.ny / 2 - 1;  // coarse centre extent
  const int per = ct * cs;  // batch * per < 2^31 (batch <= 64 slots of at most 4095^2 / 4 values)
  const int total = batch * per;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int b = t / per;
    const int rem = t - b * per;
    const int s = rem / ct, tt = rem - s * ct;
    const T* f = gf + (int64_t)b * stride;
    const int J = 2 * s + 1, I = 2 * tt + 1;
    const int c = J * ncol + I;
    const T v = f[c]
                + xscale(f[c + 1] + f[c + ncol] + f[c - 1] + f[c - ncol], 0.5f)
                + xscale(f[c + ncol + 1] + f[c - ncol + 1] + f[c - ncol - 1] + f[c + ncol - 1], 0.25f);
    gc[(int64_t)b * stride + (int64_t)(g.ny / 4 + s) * ncol + g.nx / 4 + tt] = v;
  }
}

// Multilevel curl! (fluid-ops.jl:138-182); bc == nullptr means a zero ring.  One block row per
// flux row: blockIdx.y runs over the batch's rows (ny rows of qx, then ny + 1 rows of qy), so
// an element's indices need no division.
template <typename T>
__global__ void k_curl(Geometry g, const T* __restrict__ psi, const T* __restrict__ bc, T* __restrict__ q, int batch) {
  pdl_begin();
  const int nx = g.nx, ny = g.ny, ncol = nx - 1;
  const int rows = 2 * ny + 1;
  const int b = blockIdx.y / rows, row = blockIdx.y - b * rows;
  const T* p = psi + (int64_t)b * g.nG;
  const T* c = bc ? bc + (int64_t)b * g.nbc : nullptr;
  T* qb = q + (int64_t)b * g.nq;
#define BC(i) (c ? c[(i)] : T(0))
  if (row < ny) {
    const int J = row;
    for (int I = blockIdx.x * blockDim.x + threadIdx.x; I <= nx; I += gridDim.x * blockDim.x) {
      T v;
      if (I == 0) v = BC(g.L + J + 1) - BC(g.L + J);
      else if (I == nx) v = BC(g.R + J + 1) - BC(g.R + J);
      else if (J == 0) v = p[I - 1] - BC(g.B + I);
      else if (J == ny - 1) v = BC(g.T + I) - p[(ny - 2) * ncol + I - 1];
      else v = p[J * ncol + I - 1] - p[(J - 1) * ncol + I - 1];
      qb[J * (nx + 1) + I] = v;
    }
  } else {
    const int J = row - ny;
    for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < nx; I += gridDim.x * blockDim.x) {
      T v;
      if (J == 0) v = BC(g.B + I) - BC(g.B + I + 1);
      else if (J == ny) v = BC(g.T + I) - BC(g.T + I + 1);
      else if (I == 0) v = BC(g.L + J) - p[(J - 1) * ncol];
      else if (I == nx - 1) v = p[(J - 1) * ncol + nx - 2] - BC(g.R + J);
      else v = p[(J - 1) * ncol + I - 1] - p[(J - 1) * ncol + I];
      qb[g.nu + J * nx + I] = v;
    }
  }
#undef BC
}

// rot! = C^T (fluid-ops.jl:117-129)
template <typename T>
__global__ void k_rot(Geometry g, const T* __restrict__ q, T* __restrict__ gam, int batch) {
  const int nx = g.nx, ncol = nx - 1;
  const int64_t total = (int64_t)batch * g.nG;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(t / g.nG), e = (int)(t - (int64_t)b * g.nG);
    const int J = e / ncol, I = e - J * ncol;
    const T* qx = q + (int64_t)b * g.nq;
    const T* qy = qx + g.nu;
    gam[t] = (qx[J * (nx + 1) + I + 1] - qx[(J + 1) * (nx + 1) + I + 1])
             + (qy[(J + 1) * nx + I + 1] - qy[(J + 1) * nx + I]);
  }
}

// ---- nonlinear term + explicit right-hand side (cnab/ops.jl:151-167, fluid-ops.jl:277-401,
//      cnab/timestepping.jl:54-67) ----------------------------------------------------------
template <typename T>
struct LevelView {
  const T* qx; const T* qy; const T* G; const T* bc;
  T q0x, q0y;
  int nx, ny, ncol;
  // avg_flux!: Qx at (Jq in 1..ny-1, Iq in 0..nx), Qy at (Jq in 0..ny, Iq in 1..nx-1)
  __device__ __forceinline__ T Qx(int Jq, int Iq) const {
    return xscale((((qx[Jq * (nx + 1) + Iq] + qx[(Jq - 1) * (nx + 1) + Iq]) + q0x) + q0x), 0.5f);
  }
  __device__ __forceinline__ T Qy(int Jq, int Iq) const {
    return xscale((((qy[Jq * nx + Iq] + qy[Jq * nx + Iq - 1]) + q0y) + q0y), 0.5f);
  }
  __device__ __forceinline__ T Gm(int J, int I) const { return G[J * ncol + I]; }
};

// fqx at (Jf, If), If in 1..nx-1 (direct_product_loops!, fluid-ops.jl:329-362)
template <typename T>
__device__ __forceinline__ T fqx_at(const Geometry& g, const LevelView<T>& v, int Jf, int If, T qyHi, T qyLo) {
  if (Jf == 0) return xscale(qyHi * v.Gm(0, If - 1) + qyLo * v.bc[g.B + If], 0.5f);
  if (Jf == v.ny - 1) return xscale(qyLo * v.Gm(v.ny - 2, If - 1) + qyHi * v.bc[g.T + If], 0.5f);
  return xscale(qyHi * v.Gm(Jf, If - 1) + qyLo * v.Gm(Jf - 1, If - 1), 0.5f);
}
// fqy at (Jf, If), Jf in 1..ny-1 (fluid-ops.jl:365-398); qxHi = Qx(Jf, If+1), qxLo = Qx(Jf, If)
template <typename T>
__device__ __forceinline__ T fqy_at(const Geometry& g, const LevelView<T>& v, int Jf, int If, T qxHi, T qxLo) {
  if (If == 0) return xscale(qxHi * v.Gm(Jf - 1, 0) + qxLo * v.bc[g.L + Jf], -0.5f);
  if (If == v.nx - 1) return xscale(qxLo * v.Gm(Jf - 1, v.nx - 2) + qxHi * v.bc[g.R + Jf], -0.5f);
  return xscale(qxHi * v.Gm(Jf - 1, If) + qxLo * v.Gm(Jf - 1, If - 1), -0.5f);
}

// Nonlinear term and CN right-hand side of every level (Nonlinear/RhsForce, timestepping.jl:
// 31-66; avg_flux! fluid-ops.jl:276-301, direct_product! :303-398, rot!): one block per tile of
// kNTY x kNTX cells.  The averaged fluxes (Qx, Qy) and the flux products (fqx, fqy) the tile's
// cells share are formed once into shared memory, then each cell combines its four products;
// every value is the same expression as a per-cell evaluation would form.
constexpr int kNTX = 32, kNTY = 8;
template <typename T>
__global__ void __launch_bounds__(kNTX * kNTY) k_nonlin_rhs(Geometry g, NonlinArgs<T> a) {
  pdl_begin();
  __shared__ T sQy[kNTY + 2][kNTX];   // Qy(J0 + r, I0 + 1 + c)
  __shared__ T sQx[kNTY][kNTX + 2];   // Qx(J0 + 1 + r, I0 + c)
  __shared__ T sFx[kNTY + 1][kNTX];   // fqx(J0 + r, I0 + 1 + c)
  __shared__ T sFy[kNTY][kNTX + 1];   // fqy(J0 + 1 + r, I0 + c)
  __shared__ T sK[6];                 // the tile level's q0x, q0y, 1/hc^2, alpha; dt beta0, dt beta1
  const int nx = g.nx, ny = g.ny, ncol = nx - 1, nrow = ny - 1;
  const int ne = 2 * ncol + 2 * nrow;
  const int tx = (ncol + kNTX - 1) / kNTX, ty = (nrow + kNTY - 1) / kNTY;
  const int ntiles = g.nlev * tx * ty;
  const int tid = threadIdx.x, cr = tid / kNTX, cc = tid % kNTX;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int l = tile / (tx * ty), rem = tile - l * tx * ty;
    const int J0 = (rem / tx) * kNTY, I0 = (rem % tx) * kNTX;
    LevelView<T> v;
    v.qx = a.q + (int64_t)l * g.nq;
    v.qy = v.qx + g.nu;
    v.G = a.gamma + (int64_t)l * g.nG;
    v.bc = a.bcn + (int64_t)l * g.nbc;
    // the level's constants, converted once per tile (a double-to-float-float conversion costs
    // FP64 operations, which GB300 runs at 1/64 of its FP32 rate)
    if (tid < 6) {
      const double kv = tid == 0 ? a.q0[2 * l]
                      : tid == 1 ? a.q0[2 * l + 1]
                      : tid == 2 ? a.inv_hc2[l]
                      : tid == 3 ? (a.alpha ? a.alpha[l] : 0.0)
                      : tid == 4 ? a.dtb0 : a.dtb1;
      sK[tid] = (T)kv;
    }
    __syncthreads();
    v.q0x = sK[0];
    v.q0y = sK[1];
    v.nx = nx; v.ny = ny; v.ncol = ncol;
    // averaged fluxes: Qy rows 0..ny, columns 1..nx-1; Qx rows 1..ny-1, columns 0..nx
    for (int i = tid; i < (kNTY + 2) * kNTX; i += kNTX * kNTY) {
      const int r = i / kNTX, c = i % kNTX, Jq = J0 + r, Iq = I0 + 1 + c;
      if (Jq <= ny && Iq <= nx - 1) sQy[r][c] = v.Qy(Jq, Iq);
    }
    for (int i = tid; i < kNTY * (kNTX + 2); i += kNTX * kNTY) {
      const int r = i / (kNTX + 2), c = i % (kNTX + 2), Jq = J0 + 1 + r, Iq = I0 + c;
      if (Jq <= ny - 1 && Iq <= nx) sQx[r][c] = v.Qx(Jq, Iq);
    }
    __syncthreads();
    // flux products: fqx rows 0..ny-1, columns 1..nx-1; fqy rows 1..ny-1, columns 0..nx-1
    for (int i = tid; i < (kNTY + 1) * kNTX; i += kNTX * kNTY) {
      const int r = i / kNTX, c = i % kNTX, Jf = J0 + r, If = I0 + 1 + c;
      if (Jf <= ny - 1 && If <= nx - 1) sFx[r][c] = fqx_at(g, v, Jf, If, sQy[r + 1][c], sQy[r][c]);
    }
    for (int i = tid; i < kNTY * (kNTX + 1); i += kNTX * kNTY) {
      const int r = i / (kNTX + 1), c = i % (kNTX + 1), Jf = J0 + 1 + r, If = I0 + c;
      if (Jf <= ny - 1 && If <= nx - 1) sFy[r][c] = fqy_at(g, v, Jf, If, sQx[r][c + 1], sQx[r][c]);
    }
    __syncthreads();
    const int J = J0 + cr, I = I0 + cc;
    if (J < nrow && I < ncol) {
      const int64_t t = (int64_t)l * g.nG + (int64_t)J * ncol + I;
      const T fx_lo = sFx[cr][cc];       // fqx[J,   I+1]
      const T fx_hi = sFx[cr + 1][cc];   // fqx[J+1, I+1]
      const T fy_r = sFy[cr][cc + 1];    // fqy[J+1, I+1]
      const T fy_l = sFy[cr][cc];        // fqy[J+1, I]
      const T nl = ((fx_lo - fx_hi) + (fy_r - fy_l)) * sK[2];
      a.nl_new[t] = nl;
      T r = sK[4] * nl;
      r = r + sK[5] * a.nl_old[t];
      if (a.alpha) {
        // A_l gamma = gamma - alpha_l (4 gamma - neighbours), zero outside the array
        const T gc = v.Gm(J, I);
        T lap = xscale(gc, 4.0f);
        if (I > 0) lap -= v.Gm(J, I - 1);
        if (I < ncol - 1) lap -= v.Gm(J, I + 1);
        if (J > 0) lap -= v.Gm(J - 1, I);
        if (J < nrow - 1) lap -= v.Gm(J + 1, I);
        r = (gc - sK[3] * lap) + r;
      }
      const T* ed = a.edges + (int64_t)l * ne;
      T edge = T(0);
      if (J == 0) edge += ed[I];
      if (J == nrow - 1) edge += ed[ncol + I];
      if (I == 0) edge += ed[2 * ncol + J];
      if (I == ncol - 1) edge += ed[2 * ncol + nrow + J];
      a.rhs[t] = r + edge;
    }
    __syncthreads();
  }
}

// Rings of the trial step (cnab/timestepping.jl:42-57): bcn[l] = 0.25 * get_bc(gamma[l+1]) for
// l < nlev-1 (zero on the coarsest level) and the accumulated rhsbc edge vectors
// edges[l] = sum_{l' = l}^{nlev-2} fac[l'] * get_bc(gamma[l'+1]) on the four edges.
template <typename T>
__global__ void k_trial_rings(Geometry g, const T* __restrict__ gamma, T* __restrict__ bcn, T* __restrict__ edges,
                              const double* __restrict__ fac, int accumulate) {
  pdl_begin();
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const int ne = 2 * ncol + 2 * nrow;
  const int nl = g.nlev;
  const int64_t nb_total = (int64_t)nl * g.nbc;
  const int64_t total = nb_total + (int64_t)nl * ne;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    if (t < nb_total) {
      const int l = (int)(t / g.nbc), idx = (int)(t - (int64_t)l * g.nbc);
      bcn[t] = (l < nl - 1) ? xscale(ring_value(g, gamma + (int64_t)(l + 1) * g.nG, idx), 0.25f) : T(0);
    } else {
      const int64_t u = t - nb_total;
      const int l = (int)(u / ne), e = (int)(u - (int64_t)l * ne);
      int ridx;
      if (e < ncol) ridx = g.B + 1 + e;
      else if (e < 2 * ncol) ridx = g.T + 1 + (e - ncol);
      else if (e < 2 * ncol + nrow) ridx = g.L + 1 + (e - 2 * ncol);
      else ridx = g.R + 1 + (e - 2 * ncol - nrow);
      T acc = T(0);
      if (accumulate) {
        for (int lp = nl - 2; lp >= l; --lp) acc += (T)fac[lp] * ring_value(g, gamma + (int64_t)(lp + 1) * g.nG, ridx);
      } else if (l < nl - 1) {
        acc = (T)fac[l] * ring_value(g, gamma + (int64_t)(l + 1) * g.nG, ridx);
      }
      edges[u] = acc;
    }
  }
}

// One Runge-Kutta-Chebyshev stage, elementwise over n values:
//   Y = a0 Y0 + a1 Ym1 + a2 Ym2 + c1 (G - Ym1) + c0 F0,   G = Ym1 + F(Ym1)
// (Ym2 may be null when a2 = 0; Y may alias Ym2).  With store_f0, F0 = G - Ym1 is also written.
__global__ void k_rkc_stage(int64_t n, double* __restrict__ Y, const double* __restrict__ Y0, const double* Ym1,
                            const double* Ym2, const double* __restrict__ G, double* F0, double a0, double a1,
                            double a2, double c1, double c0, int store_f0) {
  pdl_begin();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double ym1 = Ym1[i];
    const double f = G[i] - ym1;
    if (store_f0) F0[i] = f;
    double y = a0 * Y0[i] + a1 * ym1 + c1 * f;
    if (Ym2) y += a2 * Ym2[i];
    if (!store_f0) y += c0 * F0[i];
    Y[i] = y;
  }
}

template <typename T>
__global__ void k_fill(T* p, T v, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) p[t] = v;
}
template <typename T>
__global__ void k_axpby(T* y, const T* x, T a, T b, int64_t n) {
  pdl_begin();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    y[t] = a * x[t] + b * y[t];
}

}  // namespace

template <typename T>
cudaError_t get_bc(const Geometry& g, const T* r, T* bc, int batch, T extra, cudaStream_t s) {
  return launch_k(k_get_bc<T>, dim3(blocks_for((int64_t)batch * g.nbc)), dim3(kThreads), 0, s, g, r, bc, batch, extra);
}
template <typename T>
cudaError_t apply_bc(const Geometry& g, T* r, const T* bc, T fac, int batch, cudaStream_t s) {
  cudaError_t e = launch_k(k_apply_bc_rows<T>, dim3(blocks_for((int64_t)batch * (g.nx - 1))), dim3(kThreads), 0, s, g, r, bc, fac, batch);
  if (e != cudaSuccess) return e;
  return launch_k(k_apply_bc_cols<T>, dim3(blocks_for((int64_t)batch * (g.ny - 1))), dim3(kThreads), 0, s, g, r, bc, fac, batch);
}
template <typename T>
cudaError_t coarsify(const Geometry& g, T* gc, const T* gf, int batch, int64_t stride, cudaStream_t s) {
  return launch_k(k_coarsify<T>, dim3(blocks_for((int64_t)batch * (g.nx / 2 - 1) * (g.ny / 2 - 1))), dim3(kThreads), 0, s, g, gc, gf, batch, stride);
}
template <typename T>
cudaError_t curl(const Geometry& g, const T* psi, const T* bc, T* q, int batch, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  const int64_t rows = (int64_t)batch * (2 * g.ny + 1);
  if (rows > 65535) {
    for (int b = 0; b < batch; ++b) {
      cudaError_t e = curl<T>(g, psi + (int64_t)b * g.nG, bc ? bc + (int64_t)b * g.nbc : nullptr, q + (int64_t)b * g.nq, 1, s);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  const dim3 grid((g.nx + 1 + kThreads - 1) / kThreads, (unsigned)rows);
  return launch_k(k_curl<T>, grid, dim3(kThreads), 0, s, g, psi, bc, q, batch);
}
template <typename T>
cudaError_t rot(const Geometry& g, const T* q, T* gam, int batch, cudaStream_t s) {
  k_rot<T><<<blocks_for((int64_t)batch * g.nG), kThreads, 0, s>>>(g, q, gam, batch);
  return cudaGetLastError();
}
template <typename T>
cudaError_t nonlin_rhs(const Geometry& g, const NonlinArgs<T>& a, cudaStream_t s) {
  ProfScope prof(kClassNonlin, s);
  const int tiles = g.nlev * ((g.nx - 1 + kNTX - 1) / kNTX) * ((g.ny - 1 + kNTY - 1) / kNTY);
  return launch_k(k_nonlin_rhs<T>, dim3(tiles < 65535 * 8 ? tiles : 65535 * 8), dim3(kNTX * kNTY), 0, s, g, a);
}
template <typename T>
cudaError_t trial_rings(const Geometry& g, const T* gamma, T* bcn, T* edges, const double* fac, cudaStream_t s,
                        bool accumulate) {
  const int64_t n = (int64_t)g.nlev * g.nbc + (int64_t)g.nlev * (2 * (g.nx - 1) + 2 * (g.ny - 1));
  return launch_k(k_trial_rings<T>, dim3(blocks_for(n)), dim3(kThreads), 0, s, g, gamma, bcn, edges, fac,
                  accumulate ? 1 : 0);
}
cudaError_t rkc_stage(int64_t n, double* Y, const double* Y0, const double* Ym1, const double* Ym2, const double* G,
                      double* F0, double a0, double a1, double a2, double c1, double c0, bool store_f0, cudaStream_t s) {
  return launch_k(k_rkc_stage, dim3(blocks_for(n)), dim3(kThreads), 0, s, n, Y, Y0, Ym1, Ym2, G, F0, a0, a1, a2, c1, c0,
                  store_f0 ? 1 : 0);
}

template <typename T>
cudaError_t fill(T* p, T v, int64_t n, cudaStream_t s) {
  k_fill<T><<<blocks_for(n), kThreads, 0, s>>>(p, v, n);
  return cudaGetLastError();
}
template <typename T>
cudaError_t axpby(T* y, const T* x, T a, T b, int64_t n, cudaStream_t s) {
  return launch_k(k_axpby<T>, dim3(blocks_for(n)), dim3(kThreads), 0, s, y, x, a, b, n);
}

#define IB_INST(T)                                                                                   \
  template cudaError_t get_bc<T>(const Geometry&, const T*, T*, int, T, cudaStream_t);               \
  template cudaError_t apply_bc<T>(const Geometry&, T*, const T*, T, int, cudaStream_t);             \
  template cudaError_t coarsify<T>(const Geometry&, T*, const T*, int, int64_t, cudaStream_t);       \
  template cudaError_t curl<T>(const Geometry&, const T*, const T*, T*, int, cudaStream_t);          \
  template cudaError_t rot<T>(const Geometry&, const T*, T*, int, cudaStream_t);                     \
  template cudaError_t nonlin_rhs<T>(const Geometry&, const NonlinArgs<T>&, cudaStream_t);           \
  template cudaError_t trial_rings<T>(const Geometry&, const T*, T*, T*, const double*, cudaStream_t, bool); \
  template cudaError_t fill<T>(T*, T, int64_t, cudaStream_t);                                        \
  template cudaError_t axpby<T>(T*, const T*, T, T, int64_t, cudaStream_t);
IB_INST(double)
IB_INST(df64)
#undef IB_INST

}  // namespace ib
