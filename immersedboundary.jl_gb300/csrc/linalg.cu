// Dense FP64 linear algebra for the static-body Schur complement.
//
// The reference assembles B column by column and takes `inv(Bmat)` (LAPACK getrf/getri,
// src/streamfcn/cnab/ops.jl:79-97), then applies it with a dense matvec every step
// (ops.jl:97 via BoundaryForcer, cnab/timestepping.jl:106-120).  B is not exactly symmetric
// (multilevel coupling), so a Cholesky factor would not reproduce it; this file inverts B on
// the device with a blocked Gauss-Jordan sweep (64-wide pivot blocks, partial pivoting inside
// each block) whose rank-64 updates are tiled FP64 GEMMs.
#include "ib_common.cuh"

namespace ib {

namespace {

constexpr int NB = 64;  // pivot block width

// y = A x, A row-major n x n; one warp per row, lanes stride the row, fixed-order reduction.
__global__ void k_gemv_rm(const double* __restrict__ A, const double* __restrict__ x, double* __restrict__ y, int n) {
  pdl_begin();
  const int lane = threadIdx.x & 31;
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (row >= n) return;
  const double* a = A + row * (int64_t)n;
  double acc = 0.0;
  for (int j = lane; j < n; j += 32) acc = fma(a[j], x[j], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) y[row] = acc;
}

__global__ void k_transpose(const double* __restrict__ in, double* __restrict__ out, int rows, int cols) {
  __shared__ double tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = by + j, c = bx + threadIdx.x;
    if (r < rows && c < cols) tile[j][threadIdx.x] = in[(int64_t)r * cols + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int c = bx + j, r = by + threadIdx.x;
    if (r < rows && c < cols) out[(int64_t)c * rows + r] = tile[threadIdx.x][j];
  }
}

// In-place Gauss-Jordan inverse of the nb x nb diagonal block P = A[K,K] (column-major A with
// leading dimension n), written to Pinv (column-major nb x nb); also copies the column
// panel Cp = A[:, K] (n x nb, column-major).  One block of 256 threads.
__global__ void k_block_inverse(const double* __restrict__ A, int n, int k0, int nbk, double* __restrict__ Pinv,
                                double* __restrict__ Cp, int* __restrict__ status) {
  __shared__ double P[NB][NB + 1];  // P[row][col]
  __shared__ int perm[NB];
  __shared__ int piv;
  const int t = threadIdx.x;
  for (int e = t; e < NB * NB; e += blockDim.x) {
    const int r = e % NB, c = e / NB;
    P[r][c] = (r < nbk && c < nbk) ? A[(int64_t)(k0 + c) * n + k0 + r] : (r == c ? 1.0 : 0.0);
  }
  for (int64_t e = t; e < (int64_t)n * nbk; e += blockDim.x) {
    const int c = (int)(e / n), r = (int)(e - (int64_t)c * n);
    Cp[(int64_t)c * n + r] = A[(int64_t)(k0 + c) * n + r];
  }
  __syncthreads();
  for (int k = 0; k < nbk; ++k) {
    if (t < 32) {  // pivot search in column k, rows k..nbk-1
      double best = -1.0;
      int bi = k;
      for (int r = k + t; r < nbk; r += 32) {
        const double v = fabs(P[r][k]);
        if (v > best || (v == best && r < bi)) { best = v; bi = r; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (t == 0) {
        piv = bi;
        perm[k] = bi;
        if (!(best > 0.0) || !isfinite(best)) atomicExch(status, 1);
      }
    }
    __syncthreads();
    const int p = piv;
    if (p != k)
      for (int c = t; c < nbk; c += blockDim.x) {
        const double tmp = P[k][c];
        P[k][c] = P[p][c];
        P[p][c] = tmp;
      }
    __syncthreads();
    const double d = P[k][k];
    const double inv = 1.0 / d;
    __syncthreads();
    // row k: scale, with the diagonal slot holding the inverse's entry
    for (int c = t; c < nbk; c += blockDim.x) P[k][c] = (c == k) ? inv : P[k][c] * inv;
    __syncthreads();
    // eliminate the other rows
    for (int e = t; e < nbk * nbk; e += blockDim.x) {
      const int r = e % nbk, c = e / nbk;
      if (r != k) {
        const double f = P[r][k];
        if (c == k) continue;
        P[r][c] -= f * P[k][c];
      }
    }
    __syncthreads();
    for (int r = t; r < nbk; r += blockDim.x)
      if (r != k) P[r][k] = -P[r][k] * inv;
    __syncthreads();
  }
  // undo the row interchanges as column interchanges, in reverse order
  for (int k = nbk - 1; k >= 0; --k) {
    const int p = perm[k];
    if (p != k)
      for (int r = t; r < nbk; r += blockDim.x) {
        const double tmp = P[r][k];
        P[r][k] = P[r][p];
        P[r][p] = tmp;
      }
    __syncthreads();
  }
  for (int e = t; e < nbk * nbk; e += blockDim.x) {
    const int r = e % nbk, c = e / nbk;
    Pinv[(int64_t)c * nbk + r] = P[r][c];
  }
}

// Y = Pinv * A[K, :] for columns outside K; Y[:, K] = Pinv.  Y is column-major nbk x n.
__global__ void k_row_panel(const double* __restrict__ A, int n, int k0, int nbk, const double* __restrict__ Pinv,
                            double* __restrict__ Y) {
  __shared__ double Ps[NB][NB + 1];
  for (int e = threadIdx.x; e < nbk * nbk; e += blockDim.x) Ps[e % nbk][e / nbk] = Pinv[e];
  __syncthreads();
  const int64_t total = (int64_t)n * nbk;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / nbk), r = (int)(e - (int64_t)j * nbk);
    double v;
    if (j >= k0 && j < k0 + nbk) {
      v = Ps[r][j - k0];
    } else {
      const double* col = A + (int64_t)j * n + k0;
      v = 0.0;
      for (int k = 0; k < nbk; ++k) v = fma(Ps[r][k], col[k], v);
    }
    Y[(int64_t)j * nbk + r] = v;
  }
}

// A[i, j] <- (i in K) ? Y[i-k0, j] : (j in K ? 0 : A[i,j]) - sum_k Cp[i,k] Y[k,j]
// 64x64 output tile per block, 256 threads with 4x4 outputs each.
__global__ void __launch_bounds__(256) k_gj_update(double* __restrict__ A, int n, int k0, int nbk,
                                                   const double* __restrict__ Cp, const double* __restrict__ Y) {
  constexpr int KC = 32;              // k chunk held in shared memory
  __shared__ double Xs[KC][64 + 1];  // Xs[k][i]
  __shared__ double Ys[KC][64 + 1];  // Ys[k][j]
  const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
  const int t = threadIdx.x;
  const int ti = (t % 16) * 4, tj = (t / 16) * 4;
  double acc[4][4] = {};
  for (int kc = 0; kc < nbk; kc += KC) {
    for (int e = t; e < KC * 64; e += 256) {
      const int k = e / 64, r = e % 64;
      Xs[k][r] = (kc + k < nbk && i0 + r < n) ? Cp[(int64_t)(kc + k) * n + i0 + r] : 0.0;
    }
    for (int e = t; e < KC * 64; e += 256) {
      const int c = e / KC, k = e % KC;
      Ys[k][c] = (kc + k < nbk && j0 + c < n) ? Y[(int64_t)(j0 + c) * nbk + kc + k] : 0.0;
    }
    __syncthreads();
    for (int k = 0; k < KC; ++k) {
      double xa[4], yb[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) { xa[u] = Xs[k][ti + u]; yb[u] = Ys[k][tj + u]; }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(xa[u], yb[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = i0 + ti + u, j = j0 + tj + v;
      if (i >= n || j >= n) continue;
      double* a = A + (int64_t)j * n + i;
      if (i >= k0 && i < k0 + nbk) {
        *a = Y[(int64_t)j * nbk + (i - k0)];
      } else {
        const double base = (j >= k0 && j < k0 + nbk) ? 0.0 : *a;
        *a = base - acc[u][v];
      }
    }
}

}  // namespace

// y = A x for row-major A with an even row length (16-byte aligned rows): two warps per row,
// each over one half of the row with 16-byte loads and four independent partial sums per lane
// (more loads in flight than one warp per row gives, with ~n/16 warps for the whole GPU),
// combined in a fixed order: lanes, then the two halves.
__global__ void k_gemv_rm2(const double* __restrict__ A, const double* __restrict__ x, double* __restrict__ y, int n) {
  pdl_begin();
  __shared__ double part[4][2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;  // 4 warps: 2 rows x 2 halves
  const int64_t row = (int64_t)blockIdx.x * 2 + (w >> 1);
  const int half = w & 1;
  const int n2 = n / 2;
  const int h0 = half ? n2 / 2 : 0, h1 = half ? n2 : n2 / 2;  // double2 index range of this half
  double t = 0.0;
  if (row < n) {
    const double2* a = reinterpret_cast<const double2*>(A + row * (int64_t)n);
    const double2* xv = reinterpret_cast<const double2*>(x);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    int j = h0 + lane;
    for (; j + 96 < h1; j += 128) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const double2 av = __ldg(&a[j + 32 * u]), xw = __ldg(&xv[j + 32 * u]);
        acc[u] = fma(av.x, xw.x, acc[u]);
        acc[u] = fma(av.y, xw.y, acc[u]);
      }
    }
    for (int u = 0; j < h1; j += 32, ++u) {
      const double2 av = __ldg(&a[j]), xw = __ldg(&xv[j]);
      acc[u & 3] = fma(av.x, xw.x, acc[u & 3]);
      acc[u & 3] = fma(av.y, xw.y, acc[u & 3]);
    }
    t = (acc[0] + acc[1]) + (acc[2] + acc[3]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  if (lane == 0) part[w >> 1][half] = t;
  __syncthreads();
  if (threadIdx.x < 2) {
    const int64_t r = (int64_t)blockIdx.x * 2 + threadIdx.x;
    if (r < n) y[r] = part[threadIdx.x][0] + part[threadIdx.x][1];
  }
}

cudaError_t gemv_rowmajor(const double* A, const double* x, double* y, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t threads = (int64_t)n * 32;
  if (n % 2 == 0 && ((uintptr_t)A % 16) == 0 && ((uintptr_t)x % 16) == 0) {
    return launch_k(k_gemv_rm2, dim3((n + 1) / 2), dim3(128), 0, s, A, x, y, n);
  }
  k_gemv_rm<<<(int)((threads + 255) / 256), 256, 0, s>>>(A, x, y, n);
  return cudaGetLastError();
}

cudaError_t transpose(const double* in, double* out, int rows, int cols, cudaStream_t s) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  k_transpose<<<grid, block, 0, s>>>(in, out, rows, cols);
  return cudaGetLastError();
}

size_t invert_workspace_bytes(int n) {
  // Pinv (NB*NB) + Cp (n*NB) + Y (NB*n)
  return sizeof(double) * ((size_t)NB * NB + 2 * (size_t)n * NB);
}

cudaError_t invert_inplace(double* A, int n, double* work, int* status, cudaStream_t s) {
  double* Pinv = work;
  double* Cp = Pinv + NB * NB;
  double* Y = Cp + (size_t)n * NB;
  const dim3 tiles((n + 63) / 64, (n + 63) / 64);
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int nbk = (n - k0 < NB) ? n - k0 : NB;
    k_block_inverse<<<1, 256, 0, s>>>(A, n, k0, nbk, Pinv, Cp, status);
    const int64_t tot = (int64_t)n * nbk;
    k_row_panel<<<(int)((tot + 255) / 256 > 4096 ? 4096 : (tot + 255) / 256), 256, 0, s>>>(A, n, k0, nbk, Pinv, Y);
    k_gj_update<<<tiles, 256, 0, s>>>(A, n, k0, nbk, Cp, Y);
  }
  return cudaGetLastError();
}

}  // namespace ib
