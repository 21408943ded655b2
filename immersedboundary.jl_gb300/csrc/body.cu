// Immersed-body operators: regularized delta weights, E (gather), E^T (scatter), forces.
//
// Restates src/streamfcn/structure-ops.jl:24-171 and src/streamfcn/states.jl:53-84.
// Every reduction has a fixed order (no floating-point atomics), so results are identical
// from run to run.
#include "ib_common.cuh"

namespace ib {

namespace {

// E (structure-ops.jl:88-105): one warp per (point, component, column).
template <typename T>
__global__ void k_reg_gather(Geometry g, const T* __restrict__ q, const double* __restrict__ q0v, const int* __restrict__ body_idx,
                             const double* __restrict__ weight, int nb, double* __restrict__ fb, int ncols,
                             int64_t qstride, int64_t fstride) {
  pdl_begin();
  const int lane = threadIdx.x & 31;
  const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t total = (int64_t)ncols * 2 * nb;
  if (wid >= total) return;
  const int col = (int)(wid / (2 * nb));
  const int rem = (int)(wid - (int64_t)col * 2 * nb);
  const int c = rem / nb, k = rem - c * nb;
  const int i0 = body_idx[2 * k] - kSupp - 1, j0 = body_idx[2 * k + 1] - kSupp - 1;
  const T* qc = q + (int64_t)col * qstride + (c == 0 ? 0 : g.nu);
  const int pitch = (c == 0) ? g.nx + 1 : g.nx;
  const double q0 = q0v ? q0v[c] : 0.0;
  const double* w = weight + ((int64_t)k * 2 + c) * kWin2;
  double acc = 0.0;
  for (int e = lane; e < kWin2; e += 32) {
    const int b = e / kWin, a = e - b * kWin;
    const double qv = (double)qc[(j0 + b) * pitch + i0 + a] + q0;
    acc = fma(qv, w[e], acc);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) fb[(int64_t)col * fstride + k + c * nb] = acc;
}

// E^T on tiles (structure-ops.jl:63-86).  A block owns a 16x16 tile of one flux component,
// collects, in point order, the points whose 13x13 window meets the tile, then each thread
// accumulates its face over that list: the reference's k-ordered sum, without atomics.
constexpr int kTile = 16;
constexpr int kChunk = 512;

template <typename T>
__global__ void __launch_bounds__(256) k_reg_scatter_tiles(Geometry g, const double* __restrict__ f,
                                                           const int* __restrict__ body_idx,
                                                           const double* __restrict__ weight, int nb, T* __restrict__ q,
                                                           int tiles_x0, int tiles_y0, int tiles_x1, int tiles_y1,
                                                           int* __restrict__ status, const int* __restrict__ box) {
  pdl_begin();
  __shared__ int list[kChunk];
  __shared__ int count;
  __shared__ int warp_counts[8];
  const int ntx = tiles_x1 - tiles_x0, nty = tiles_y1 - tiles_y0;
  const int tile = blockIdx.x % (ntx * nty);
  const int c = blockIdx.x / (ntx * nty);
  const int tx = tiles_x0 + tile % ntx, ty = tiles_y0 + tile / ntx;
  // tiles outside the box of all windows have no point: their faces are left unwritten (the
  // caller reads the flux only inside the box)
  if (box && (tx * kTile > box[1] || (tx + 1) * kTile <= box[0] || ty * kTile > box[3] || (ty + 1) * kTile <= box[2]))
    return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int fi = tx * kTile + (threadIdx.x % kTile), fj = ty * kTile + (threadIdx.x / kTile);
  const int pitch = (c == 0) ? g.nx + 1 : g.nx;
  const int rows = (c == 0) ? g.ny : g.ny + 1;
  const bool inside = fi < pitch && fj < rows;
  double acc = 0.0;
  for (int base = 0; base < nb; base += kChunk) {
    if (threadIdx.x == 0) count = 0;
    __syncthreads();
    // ordered compaction of this chunk: blocks of 256 points, warp ballots in order
    for (int sub = 0; sub < kChunk; sub += 256) {
      const int k = base + sub + threadIdx.x;
      bool hit = false;
      if (k < nb) {
        const int i0 = body_idx[2 * k] - kSupp - 1, j0 = body_idx[2 * k + 1] - kSupp - 1;
        hit = !(i0 + kWin <= tx * kTile || i0 >= (tx + 1) * kTile || j0 + kWin <= ty * kTile || j0 >= (ty + 1) * kTile);
      }
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (lane == 0) warp_counts[warp] = __popc(m);
      __syncthreads();
      int off = count;
      for (int w = 0; w < warp; ++w) off += warp_counts[w];
      if (hit) list[off + __popc(m & ((1u << lane) - 1u))] = k;
      __syncthreads();
      if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < 8; ++w) s += warp_counts[w];
        count += s;
      }
      __syncthreads();
    }
    const int n = count;
    if (inside) {
      for (int p = 0; p < n; ++p) {
        const int k = list[p];
        const int a = fi - (body_idx[2 * k] - kSupp - 1), b = fj - (body_idx[2 * k + 1] - kSupp - 1);
        if (a >= 0 && a < kWin && b >= 0 && b < kWin) {
          const double fk = f[k + c * nb];
          acc += weight[((int64_t)k * 2 + c) * kWin2 + b * kWin + a] * fk;
        }
      }
    }
    __syncthreads();
  }
  if (inside) {
    if (!isfinite(acc)) atomicExch(status, 1);
    q[(c == 0 ? 0 : g.nu) + fj * pitch + fi] = (T)acc;
  }
}

// rot of the scattered flux: full circulation array, zero outside the body box
// Face box of every point's 13x13 window, box = {i_lo, i_hi, j_lo, j_hi} (one block; the
// flux faces E^T can touch, both components).
__global__ void k_body_box(Geometry g, const int* __restrict__ body_idx, int nb, int* __restrict__ box) {
  pdl_begin();
  __shared__ int s[4][256];
  int v[4] = {1 << 30, -(1 << 30), 1 << 30, -(1 << 30)};
  for (int k = threadIdx.x; k < nb; k += blockDim.x) {
    const int i0 = body_idx[2 * k] - kSupp - 1, j0 = body_idx[2 * k + 1] - kSupp - 1;
    v[0] = min(v[0], i0);
    v[1] = max(v[1], i0 + kWin - 1);
    v[2] = min(v[2], j0);
    v[3] = max(v[3], j0 + kWin - 1);
  }
  for (int i = 0; i < 4; ++i) s[i][threadIdx.x] = v[i];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s[0][threadIdx.x] = min(s[0][threadIdx.x], s[0][threadIdx.x + o]);
      s[1][threadIdx.x] = max(s[1][threadIdx.x], s[1][threadIdx.x + o]);
      s[2][threadIdx.x] = min(s[2][threadIdx.x], s[2][threadIdx.x + o]);
      s[3][threadIdx.x] = max(s[3][threadIdx.x], s[3][threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    box[0] = max(s[0][0], 0);
    box[1] = min(s[1][0], g.nx);
    box[2] = max(s[2][0], 0);
    box[3] = min(s[3][0], g.ny);
  }
}

template <typename T>
__global__ void k_rot_box(Geometry g, const T* __restrict__ q, T* __restrict__ gam, int i_lo, int i_hi, int j_lo, int j_hi,
                          const int* __restrict__ box) {
  pdl_begin();
  const int nx = g.nx, ncol = nx - 1;
  if (box) {
    i_lo = box[0]; i_hi = box[1]; j_lo = box[2]; j_hi = box[3];
  }
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < g.nG; t += gridDim.x * blockDim.x) {
    const int J = t / ncol, I = t - J * ncol;
    T v = T(0);
    // node (J, I) touches qx faces (J, I+1), (J+1, I+1) and qy faces (J+1, I), (J+1, I+1)
    if (I + 1 >= i_lo && I <= i_hi && J + 1 >= j_lo && J <= j_hi) {
      auto QX = [&](int jj, int ii) -> T {
        return (ii >= i_lo && ii <= i_hi && jj >= j_lo && jj <= j_hi) ? q[jj * (nx + 1) + ii] : T(0);
      };
      auto QY = [&](int jj, int ii) -> T {
        return (ii >= i_lo && ii <= i_hi && jj >= j_lo && jj <= j_hi) ? q[g.nu + jj * nx + ii] : T(0);
      };
      v = (QX(J, I + 1) - QX(J + 1, I + 1)) + (QY(J + 1, I + 1) - QY(J + 1, I));
    }
    gam[t] = v;
  }
}

// unit-force columns for the Schur assembly: gam[col] = rot(E^T e_{col0+col})
template <typename T>
__global__ void k_unit_scatter_rot(Geometry g, const int* __restrict__ body_idx, const double* __restrict__ weight, int nb,
                                   int col0, int ncols, T* __restrict__ gam) {
  const int nx = g.nx, ncol = nx - 1;
  const int64_t total = (int64_t)ncols * g.nG;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int cidx = (int)(t / g.nG);
    const int e = (int)(t - (int64_t)cidx * g.nG);
    const int J = e / ncol, I = e - J * ncol;
    const int j = col0 + cidx;
    const int c = j / nb, k = j - c * nb;
    const int i0 = body_idx[2 * k] - kSupp - 1, j0 = body_idx[2 * k + 1] - kSupp - 1;
    const double* w = weight + ((int64_t)k * 2 + c) * kWin2;
    auto W = [&](int jj, int ii) -> double {
      const int a = ii - i0, b = jj - j0;
      return (a >= 0 && a < kWin && b >= 0 && b < kWin) ? w[b * kWin + a] : 0.0;
    };
    double v = 0.0;
    if (c == 0) v = W(J, I + 1) - W(J + 1, I + 1);
    else v = W(J + 1, I + 1) - W(J + 1, I);
    gam[t] = (T)v;
  }
}

__global__ void k_unit_columns(double* f, int nf, int col0, int ncols) {
  const int64_t total = (int64_t)ncols * nf;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t / nf), r = (int)(t - (int64_t)c * nf);
    f[t] = (r == col0 + c) ? 1.0 : 0.0;
  }
}

// update_stress! (states.jl:53-84): one block per body, fixed-order block reduction.
__global__ void k_update_stress(const double* __restrict__ fb, int nb, const int* __restrict__ body_start,
                                const double* __restrict__ ds, double h, double dt, double* __restrict__ out,
                                double* __restrict__ stress) {
  pdl_begin();
  __shared__ double sx[256], sy[256];
  const int body = blockIdx.x;
  const int s0 = body_start[body], s1 = body_start[body + 1], n = s1 - s0;
  double ax = 0.0, ay = 0.0;
  for (int p = threadIdx.x; p < n; p += blockDim.x) {
    const double fx = fb[s0 + p] * h / dt, fy = fb[nb + s0 + p] * h / dt;
    ax += fx;
    ay += fy;
    if (stress) {
      stress[2 * s0 + p] = fx / ds[s0 + p];
      stress[2 * s0 + n + p] = fy / ds[s0 + p];
    }
  }
  sx[threadIdx.x] = ax;
  sy[threadIdx.x] = ay;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sx[threadIdx.x] += sx[threadIdx.x + o];
      sy[threadIdx.x] += sy[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[2 * body] = 2 * sx[0];
    out[2 * body + 1] = 2 * sy[0];
  }
}

inline int nblk(int64_t n, int t = 256) {
  int64_t b = (n + t - 1) / t;
  if (b > 65535LL * 8) b = 65535LL * 8;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace

template <typename T>
cudaError_t reg_gather(const Geometry& g, const T* q, const double* q0, const int* body_idx,
                       const double* weight, int nb, double* fb, int ncols, int64_t qstride, int64_t fstride,
                       cudaStream_t s) {
  if (nb <= 0) return cudaSuccess;
  const int64_t warps = (int64_t)ncols * 2 * nb;
  return launch_k(k_reg_gather<T>, dim3(nblk(warps * 32)), dim3(256), 0, s, g, q, q0, body_idx, weight, nb, fb, ncols, qstride, fstride);
}

// The body box (in faces) is taken from the whole flux domain; tiles outside every window
// find an empty point list and write zeros.
template <typename T>
cudaError_t reg_scatter(const Geometry& g, const double* f, const int* body_idx, const double* weight, int nb, T* q,
                        int* status, cudaStream_t s) {
  const int tx = (g.nx + 1 + kTile - 1) / kTile, ty = (g.ny + 1 + kTile - 1) / kTile;
  k_reg_scatter_tiles<T><<<2 * tx * ty, 256, 0, s>>>(g, f, body_idx, weight, nb, q, 0, 0, tx, ty, status, nullptr);
  return cudaGetLastError();
}

// rot(E^T f): the scatter covers only the faces inside the box of the windows (box: 4 ints of
// device scratch, or nullptr for the whole flux domain), the rot reads only those
cudaError_t body_box(const Geometry& g, const int* body_idx, int nb, int* box, cudaStream_t s) {
  if (nb <= 0) return cudaSuccess;
  return launch_k(k_body_box, dim3(1), dim3(256), 0, s, g, body_idx, nb, box);
}

template <typename T>
cudaError_t reg_scatter_rot(const Geometry& g, const double* f, const int* body_idx, const double* weight, int nb,
                            T* qtmp, T* gam, int ncols, int64_t fstride, int* status, int* box, bool box_ready,
                            cudaStream_t s) {
  (void)ncols;
  (void)fstride;
  if (box && nb > 0) {
    cudaError_t e = box_ready ? cudaSuccess : body_box(g, body_idx, nb, box, s);
    if (e != cudaSuccess) return e;
    const int tx = (g.nx + 1 + kTile - 1) / kTile, ty = (g.ny + 1 + kTile - 1) / kTile;
    e = launch_k(k_reg_scatter_tiles<T>, dim3(2 * tx * ty), dim3(256), 0, s, g, f, body_idx, weight, nb, qtmp, 0, 0, tx, ty, status,
                 (const int*)box);
    if (e != cudaSuccess) return e;
  } else {
    cudaError_t e = reg_scatter<T>(g, f, body_idx, weight, nb, qtmp, status, s);
    if (e != cudaSuccess) return e;
    box = nullptr;
  }
  return launch_k(k_rot_box<T>, dim3(nblk(g.nG)), dim3(256), 0, s, g, (const T*)qtmp, gam, 0, g.nx, 0, g.ny,
                  (const int*)(nb > 0 ? box : nullptr));
}

template <typename T>
cudaError_t unit_scatter_rot(const Geometry& g, const int* body_idx, const double* weight, int nb, int col0, int ncols,
                             T* gam, cudaStream_t s) {
  k_unit_scatter_rot<T><<<nblk((int64_t)ncols * g.nG), 256, 0, s>>>(g, body_idx, weight, nb, col0, ncols, gam);
  return cudaGetLastError();
}

cudaError_t unit_columns(double* f, int nf, int col0, int ncols, cudaStream_t s) {
  k_unit_columns<<<nblk((int64_t)ncols * nf), 256, 0, s>>>(f, nf, col0, ncols);
  return cudaGetLastError();
}

cudaError_t update_stress_hd(const double* fb, int nb, int nbodies, const int* body_start, const double* ds, double h,
                             double dt, double* cd_cl_out, double* stress_out, cudaStream_t s) {
  return launch_k(k_update_stress, dim3(nbodies), dim3(256), 0, s, fb, nb, body_start, ds, h, dt, cd_cl_out, stress_out);
}

template cudaError_t reg_gather<double>(const Geometry&, const double*, const double*, const int*, const double*, int,
                                        double*, int, int64_t, int64_t, cudaStream_t);
template cudaError_t reg_gather<df64>(const Geometry&, const df64*, const double*, const int*, const double*, int,
                                       double*, int, int64_t, int64_t, cudaStream_t);
template cudaError_t reg_scatter<double>(const Geometry&, const double*, const int*, const double*, int, double*, int*,
                                         cudaStream_t);
template cudaError_t reg_scatter<df64>(const Geometry&, const double*, const int*, const double*, int, df64*, int*,
                                        cudaStream_t);
template cudaError_t reg_scatter_rot<double>(const Geometry&, const double*, const int*, const double*, int, double*,
                                             double*, int, int64_t, int*, int*, bool, cudaStream_t);
template cudaError_t reg_scatter_rot<df64>(const Geometry&, const double*, const int*, const double*, int, df64*,
                                            df64*, int, int64_t, int*, int*, bool, cudaStream_t);
template cudaError_t unit_scatter_rot<double>(const Geometry&, const int*, const double*, int, int, int, double*,
                                              cudaStream_t);
template cudaError_t unit_scatter_rot<df64>(const Geometry&, const int*, const double*, int, int, int, df64*,
                                             cudaStream_t);

}  // namespace ib
