// Learned warm start for the moving-body Schur CG: a small multilayer perceptron trained on
// the force histories the solver generates, with hand-written inference and training kernels.
//
//   features x = [kinematics of every body (r0x, r0y, v0x, v0y, theta, Omega), F_{n-1}, F_{n-2}]
//   target   y = F_n - (2 F_{n-1} - F_{n-2})        (the correction to linear extrapolation)
//   network  x~ = (x - mu_x) / sd_x -> tanh(W1 x~ + b1) -> ... -> W_L h + b_L = y~,
//            y = y~ * sd_y + mu_y,  warm start F_n ~ 2 F_{n-1} - F_{n-2} + y
// Weights are stored BF16 for the forward products, with FP32 master copies updated by Adam;
// every product accumulates in FP32.  Reductions (bias gradients, loss, statistics) run in a
// fixed order, so training is reproducible.
#include "ib_common.cuh"
#include "mlp.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <type_traits>

namespace ib {
namespace learn {
namespace {

constexpr int kTile = 64, kBK = 16;

template <typename T> __device__ __forceinline__ float ldf(const T* p, int64_t i);
template <> __device__ __forceinline__ float ldf<float>(const float* p, int64_t i) { return p[i]; }
template <> __device__ __forceinline__ float ldf<__nv_bfloat16>(const __nv_bfloat16* p, int64_t i) {
  return __bfloat162float(p[i]);
}

enum Epi : int { kStore = 0, kBias = 1, kBiasTanh = 2 };

// C[M x N] = op(A)[M x K] op(B)[K x N] (+ bias[n], tanh).  A is FP32, stored [M][K] (TA false)
// or [K][M] (TA true); B is FP32 or BF16, stored [K][N] (TB false) or [N][K] (TB true).
// 64 x 64 output tile per 256-thread block, 4 x 4 outputs per thread, K in steps of 16.
template <bool TA, bool TB, typename TBt, int EPI>
__global__ void __launch_bounds__(256)
k_gemm(int M, int N, int K, const float* __restrict__ A, const TBt* __restrict__ B, float* __restrict__ C,
       const float* __restrict__ bias) {
  __shared__ float As[kBK][kTile + 4];
  __shared__ float Bs[kBK][kTile + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kBK) {
    for (int e = threadIdx.x; e < kBK * kTile; e += 256) {
      const int kk = e / kTile, mm = e % kTile;
      const int m = m0 + mm, k = k0 + kk;
      float va = 0.f;
      if (m < M && k < K) va = TA ? A[(int64_t)k * M + m] : A[(int64_t)m * K + k];
      As[kk][mm] = va;
      const int n = n0 + mm;
      float vb = 0.f;
      if (n < N && k < K) vb = TB ? ldf(B, (int64_t)n * K + k) : ldf(B, (int64_t)k * N + n);
      Bs[kk][mm] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx * 4 + j;
      if (n >= N) continue;
      float v = acc[i][j];
      if (EPI != kStore) v += bias[n];
      if (EPI == kBiasTanh) v = tanhf(v);
      C[(int64_t)m * N + n] = v;
    }
  }
}

template <bool TA, bool TB, typename TBt, int EPI>
cudaError_t gemm(int M, int N, int K, const float* A, const TBt* B, float* C, const float* bias, cudaStream_t s) {
  dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
  k_gemm<TA, TB, TBt, EPI><<<grid, 256, 0, s>>>(M, N, K, A, B, C, bias);
  return cudaGetLastError();
}

// dZ = dA * (1 - A^2) (tanh)
__global__ void k_tanh_back(const float* __restrict__ a, float* __restrict__ d, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] *= 1.f - a[i] * a[i];
}

// out[n] = sum_m in[m][n] in row order (one thread per column)
__global__ void k_colsum(const float* __restrict__ in, float* __restrict__ out, int M, int N) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; ++m) s += in[(int64_t)m * N + n];
  out[n] = s;
}

// MSE: dY = 2 (Yhat - Y) / (M N); loss (one block, fixed order) into loss[0]
__global__ void k_mse(const float* __restrict__ yh, const float* __restrict__ y, float* __restrict__ dy,
                      double* __restrict__ loss, int64_t n) {
  __shared__ double part[256];
  double s = 0.0;
  const float scale = 2.f / (float)n;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const float e = yh[i] - y[i];
    dy[i] = scale * e;
    s += (double)e * (double)e;
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss[0] = part[0] / (double)n;
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int64_t n, float lr, float b1, float b2, float c1, float c2, float eps) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_to_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ o, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    o[i] = __float2bfloat16_rn(w[i]);
}

// raw features of the current step: [kin (6 per body), f1, f2] in FP32
__global__ void k_features(const double* __restrict__ kin, int nkin, const double* __restrict__ f1,
                           const double* __restrict__ f2, int nf, float* __restrict__ x) {
  const int din = nkin + 2 * nf;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < din; i += gridDim.x * blockDim.x) {
    double v;
    if (i < nkin) v = kin[i];
    else if (i < nkin + nf) v = f1[i - nkin];
    else v = f2[i - nkin - nf];
    x[i] = (float)v;
  }
}

// ring slot *next <- (raw features, F_n), then *next advances (one block; capturable, the slot
// index lives on the device)
__global__ void k_record(const float* __restrict__ x, int din, const double* __restrict__ fn, int nf,
                         float* __restrict__ xs_all, float* __restrict__ ys_all, int* __restrict__ next, int cap) {
  const int slot = *next;
  float* xs = xs_all + (int64_t)slot * din;
  float* ys = ys_all + (int64_t)slot * nf;
  for (int i = threadIdx.x; i < din + nf; i += blockDim.x) {
    if (i < din) xs[i] = x[i];
    else ys[i - din] = (float)fn[i - din];
  }
  __syncthreads();
  if (threadIdx.x == 0) *next = (slot + 1) % cap;
}

// per-column mean and standard deviation over `count` rows (fixed order, one thread per column);
// target columns are the correction to linear extrapolation
__global__ void k_stats(const float* __restrict__ xs, const float* __restrict__ ys, const int* __restrict__ rows,
                        int count, int din, int nkin, int nf, float* __restrict__ mu_x, float* __restrict__ sd_x,
                        float* __restrict__ mu_y, float* __restrict__ sd_y) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= din + nf) return;
  double s = 0.0, s2 = 0.0;
  for (int i = 0; i < count; ++i) {
    const int r = rows[i];
    double v;
    if (c < din) {
      v = xs[(int64_t)r * din + c];
    } else {
      const int k = c - din;
      const float* x = xs + (int64_t)r * din;
      v = (double)ys[(int64_t)r * nf + k] - (2.0 * x[nkin + k] - (double)x[nkin + nf + k]);
    }
    s += v;
    s2 += v * v;
  }
  const double mean = s / count;
  const double var = std::max(s2 / count - mean * mean, 0.0);
  if (c < din) { mu_x[c] = (float)mean; sd_x[c] = (float)sqrt(var); }
  else { mu_y[c - din] = (float)mean; sd_y[c - din] = (float)sqrt(var); }
}

// input scales: a (nearly) constant feature keeps unit scale.  Output scale: one value for all
// force components (their RMS standard deviation), so the loss weighs each component by its
// actual size, which is what the CG start sees.
__global__ void k_floor_scales(float* sd_x, int din, float* sd_y, int nf) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float mx = 0.f;
  for (int i = 0; i < din; ++i) mx = fmaxf(mx, sd_x[i]);
  for (int i = 0; i < din; ++i)
    if (!(sd_x[i] > 1e-6f * mx) || sd_x[i] == 0.f) sd_x[i] = 1.f;
  double v = 0.0;
  for (int i = 0; i < nf; ++i) v += (double)sd_y[i] * sd_y[i];
  const float g = v > 0.0 ? (float)sqrt(v / nf) : 1.f;
  for (int i = 0; i < nf; ++i) sd_y[i] = g;
}

// validation sums in raw units: t = target correction, q = predicted correction;
// out += (sum t q, sum q q, sum t t) (one block, fixed order)
__global__ void k_val_sums(const float* __restrict__ yb, const float* __restrict__ yh, const float* __restrict__ mu_y,
                           const float* __restrict__ sd_y, int b, int nf, double* __restrict__ out) {
  __shared__ double part[3][256];
  double tq = 0.0, qq = 0.0, tt = 0.0;
  for (int64_t i = threadIdx.x; i < (int64_t)b * nf; i += blockDim.x) {
    const int k = (int)(i % nf);
    const double t = (double)yb[i] * sd_y[k] + mu_y[k];
    const double q = (double)yh[i] * sd_y[k] + mu_y[k];
    tq += t * q;
    qq += q * q;
    tt += t * t;
  }
  part[0][threadIdx.x] = tq;
  part[1][threadIdx.x] = qq;
  part[2][threadIdx.x] = tt;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int j = 0; j < 3; ++j) part[j][threadIdx.x] += part[j][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int j = 0; j < 3; ++j) out[j] += part[j][0];
}

// minibatch rows idx[0..b): normalised features and targets
__global__ void k_denorm(const float* __restrict__ yb, const float* __restrict__ yh, const float* __restrict__ mu_y,
                         const float* __restrict__ sd_y, int b, int nf, double* __restrict__ q, double* __restrict__ t) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)b * nf;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % nf);
    t[i] = (double)yb[i] * sd_y[k] + mu_y[k];
    q[i] = (double)yh[i] * sd_y[k] + mu_y[k];
  }
}

__global__ void k_gather(const float* __restrict__ xs, const float* __restrict__ ys, const int* __restrict__ idx, int b,
                         int din, int nkin, int nf, const float* __restrict__ mu_x, const float* __restrict__ sd_x,
                         const float* __restrict__ mu_y, const float* __restrict__ sd_y, float* __restrict__ xb,
                         float* __restrict__ yb) {
  const int64_t tot = (int64_t)b * (din + nf);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / (din + nf)), c = (int)(e % (din + nf));
    const float* x = xs + (int64_t)idx[r] * din;
    if (c < din) {
      xb[(int64_t)r * din + c] = (x[c] - mu_x[c]) / sd_x[c];
    } else {
      const int k = c - din;
      const float t = ys[(int64_t)idx[r] * nf + k] - (2.f * x[nkin + k] - x[nkin + nf + k]);
      yb[(int64_t)r * nf + k] = (t - mu_y[k]) / sd_y[k];
    }
  }
}

__global__ void k_normalize(const float* __restrict__ x, const float* __restrict__ mu, const float* __restrict__ sd,
                            float* __restrict__ xn, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) xn[i] = (x[i] - mu[i]) / sd[i];
}

// warm start: fb = 2 f1 - f2 + blend * (yhat * sd_y + mu_y); an entry whose correction is not
// finite (a network far outside its training data) keeps the extrapolation, so a start never
// brings a non-finite value into the CG
__global__ void k_predict(const float* __restrict__ yh, const float* __restrict__ mu_y, const float* __restrict__ sd_y,
                          const double* __restrict__ f1, const double* __restrict__ f2, double* __restrict__ fb,
                          int nf, double blend) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x) {
    const double ex = 2.0 * f1[i] - f2[i];
    const double c = blend * ((double)yh[i] * (double)sd_y[i] + (double)mu_y[i]);
    fb[i] = isfinite(c) ? ex + c : ex;
  }
}

int blocks_for(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

}  // namespace

// --------------------------------------------------------------------------------------------
// Mlp
// --------------------------------------------------------------------------------------------
cudaError_t Mlp::init(int din_, int dout_, int hidden, int nhidden, int capacity, uint64_t seed, cudaStream_t s) {
  release();
  stream = s;
  dims.clear();
  dims.push_back(din_);
  for (int i = 0; i < nhidden; ++i) dims.push_back(hidden);
  dims.push_back(dout_);
  nl = (int)dims.size() - 1;
  woff.assign(nl, 0);
  boff.assign(nl, 0);
  int64_t off = 0;
  nweights = 0;
  for (int l = 0; l < nl; ++l) {
    woff[l] = off;
    off += (int64_t)dims[l] * dims[l + 1];
    nweights += (int64_t)dims[l] * dims[l + 1];
    boff[l] = off;
    off += dims[l + 1];
  }
  nparam = off;
  cap = capacity;
  count = 0;
  next = 0;
  trained = false;
  adam_t = 0;
  int maxw = 0;
  for (int d : dims) maxw = std::max(maxw, d);
  auto A = [&](auto** p, size_t n) -> cudaError_t {
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, std::max<size_t>(n, 16));
    if (e != cudaSuccess) return e;
    allocs.push_back(v);
    *p = (std::remove_reference_t<decltype(*p)>)v;
    return cudaMemsetAsync(v, 0, std::max<size_t>(n, 16), stream);
  };
  cudaError_t e;
#define A_(p, n) if ((e = A(&(p), (n))) != cudaSuccess) return e
  A_(master, sizeof(float) * nparam);
  A_(grad, sizeof(float) * nparam);
  A_(adam_m, sizeof(float) * nparam);
  A_(adam_v, sizeof(float) * nparam);
  A_(wbf, sizeof(__nv_bfloat16) * nparam);
  A_(xs, sizeof(float) * (size_t)cap * din_);
  A_(ys, sizeof(float) * (size_t)cap * dout_);
  A_(feat, sizeof(float) * din_);
  A_(featn, sizeof(float) * din_);
  A_(mu_x, sizeof(float) * din_);
  A_(sd_x, sizeof(float) * din_);
  A_(mu_y, sizeof(float) * dout_);
  A_(sd_y, sizeof(float) * dout_);
  A_(loss, sizeof(double) * 4);
  A_(idx, sizeof(int) * (size_t)cap);
  A_(d_next, sizeof(int));
  act.assign(nl + 1, nullptr);
  dact.assign(nl + 1, nullptr);
  for (int l = 0; l <= nl; ++l) {
    A_(act[l], sizeof(float) * (size_t)kMaxBatch * dims[l]);
    A_(dact[l], sizeof(float) * (size_t)kMaxBatch * dims[l]);
  }
  A_(ybatch, sizeof(float) * (size_t)kMaxBatch * dout_);
#undef A_
  // Xavier-uniform weights (seeded), zero biases
  std::vector<float> h(nparam, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < nl; ++l) {
    const double a = std::sqrt(6.0 / (dims[l] + dims[l + 1]));
    std::uniform_real_distribution<double> u(-a, a);
    for (int64_t i = 0; i < (int64_t)dims[l] * dims[l + 1]; ++i) h[woff[l] + i] = (float)u(rng);
  }
  // the last layer starts at zero: the untrained network predicts plain extrapolation
  std::fill(h.begin() + woff[nl - 1], h.begin() + woff[nl - 1] + (int64_t)dims[nl - 1] * dims[nl], 0.f);
  if ((e = cudaMemcpyAsync(master, h.data(), sizeof(float) * nparam, cudaMemcpyHostToDevice, stream)) != cudaSuccess)
    return e;
  std::vector<float> ones_x(din_, 1.f), ones_y(dout_, 1.f);
  if ((e = cudaMemcpyAsync(sd_x, ones_x.data(), sizeof(float) * din_, cudaMemcpyHostToDevice, stream)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(sd_y, ones_y.data(), sizeof(float) * dout_, cudaMemcpyHostToDevice, stream)) != cudaSuccess)
    return e;
  if ((e = sync_bf16()) != cudaSuccess) return e;
  return cudaStreamSynchronize(stream);
}

void Mlp::release() {
  for (void* p : allocs) cudaFree(p);
  allocs.clear();
  nl = 0;
}

cudaError_t Mlp::sync_bf16() {
  k_to_bf16<<<blocks_for(nparam), 256, 0, stream>>>(master, wbf, nparam);
  return cudaGetLastError();
}

// forward of `b` normalised rows in act[0] -> act[nl]
cudaError_t Mlp::forward(int b) {
  for (int l = 0; l < nl; ++l) {
    const int K = dims[l], N = dims[l + 1];
    const __nv_bfloat16* W = wbf + woff[l];
    const float* bias = master + boff[l];
    cudaError_t e = (l + 1 < nl) ? gemm<false, true, __nv_bfloat16, kBiasTanh>(b, N, K, act[l], W, act[l + 1], bias, stream)
                                 : gemm<false, true, __nv_bfloat16, kBias>(b, N, K, act[l], W, act[l + 1], bias, stream);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// loss and gradients (into grad) of `b` rows: act[0] inputs, ybatch targets
cudaError_t Mlp::backward(int b) {
  cudaError_t e;
  const int64_t nout = (int64_t)b * dims[nl];
  k_mse<<<1, 256, 0, stream>>>(act[nl], ybatch, dact[nl], loss, nout);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  for (int l = nl - 1; l >= 0; --l) {
    const int K = dims[l], N = dims[l + 1];
    // dact[l+1] holds dZ of layer l (the output layer is linear; hidden layers apply tanh')
    if (l + 1 < nl) {
      k_tanh_back<<<blocks_for((int64_t)b * N), 256, 0, stream>>>(act[l + 1], dact[l + 1], (int64_t)b * N);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // dW = dZ^T X  [N x K] ;  db = column sums of dZ
    if ((e = gemm<true, false, float, kStore>(N, K, b, dact[l + 1], act[l], grad + woff[l], nullptr, stream)) != cudaSuccess)
      return e;
    k_colsum<<<(N + 127) / 128, 128, 0, stream>>>(dact[l + 1], grad + boff[l], b, N);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // dX = dZ W  [b x K]
    if (l > 0) {
      if ((e = gemm<false, false, __nv_bfloat16, kStore>(b, K, N, dact[l + 1], wbf + woff[l], dact[l], nullptr, stream)) !=
          cudaSuccess)
        return e;
    }
  }
  return cudaSuccess;
}

cudaError_t Mlp::adam_step(float lr) {
  ++adam_t;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)adam_t), c2 = 1.f - std::pow(b2, (float)adam_t);
  k_adam<<<blocks_for(nparam), 256, 0, stream>>>(master, grad, adam_m, adam_v, nparam, lr, b1, b2, c1, c2, 1e-8f);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return sync_bf16();
}

cudaError_t Mlp::features(const double* kin, int nkin, const double* f1, const double* f2, int nf) {
  k_features<<<blocks_for(dims[0]), 256, 0, stream>>>(kin, nkin, f1, f2, nf, feat);
  return cudaGetLastError();
}

cudaError_t Mlp::record_enqueue(const double* fn) {
  const int din = dims[0], nf = dims[nl];
  k_record<<<1, 256, 0, stream>>>(feat, din, fn, nf, xs, ys, d_next, cap);
  return cudaGetLastError();
}

void Mlp::record_commit() {
  next = (next + 1) % cap;
  count = std::min(count + 1, cap);
}

cudaError_t Mlp::record(const double* fn) {
  cudaError_t e = record_enqueue(fn);
  if (e == cudaSuccess) record_commit();
  return e;
}

cudaError_t Mlp::predict(const double* f1, const double* f2, double* fb) {
  const int din = dims[0], nf = dims[nl];
  k_normalize<<<blocks_for(din), 256, 0, stream>>>(feat, mu_x, sd_x, act[0], din);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if ((e = forward(1)) != cudaSuccess) return e;
  k_predict<<<blocks_for(nf), 256, 0, stream>>>(act[nl], mu_y, sd_y, f1, f2, fb, nf, blend);
  return cudaGetLastError();
}

cudaError_t Mlp::train(int epochs, int batch, float lr, uint64_t seed, double* final_loss) {
  const int din = dims[0], nf = dims[nl];
  const int nkin = din - 2 * nf;
  if (count < 2 || batch < 1 || batch > kMaxBatch) return cudaErrorInvalidValue;
  cudaError_t e;
  // samples in time order; the most recent tenth is held out to validate the network and to
  // choose the blend between extrapolation and the network's correction
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = ((next - count + i) % cap + cap) % cap;
  const int nval = count >= 20 ? count / 10 : 0;
  const int ntr = count - nval;
  if ((e = cudaMemcpyAsync(idx, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice, stream)) != cudaSuccess)
    return e;
  k_stats<<<(din + nf + 127) / 128, 128, 0, stream>>>(xs, ys, idx, ntr, din, nkin, nf, mu_x, sd_x, mu_y, sd_y);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_floor_scales<<<1, 32, 0, stream>>>(sd_x, din, sd_y, nf);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  std::vector<int> perm(order.begin(), order.begin() + ntr);
  std::mt19937_64 rng(seed);
  double last = 0.0;
  for (int ep = 0; ep < epochs; ++ep) {
    std::shuffle(perm.begin(), perm.end(), rng);
    if ((e = cudaMemcpyAsync(idx, perm.data(), sizeof(int) * ntr, cudaMemcpyHostToDevice, stream)) != cudaSuccess)
      return e;
    double sum = 0.0;
    int nb = 0;
    for (int s0 = 0; s0 < ntr; s0 += batch) {
      const int b = std::min(batch, ntr - s0);
      k_gather<<<blocks_for((int64_t)b * (din + nf)), 256, 0, stream>>>(xs, ys, idx + s0, b, din, nkin, nf, mu_x, sd_x,
                                                                         mu_y, sd_y, act[0], ybatch);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      if ((e = forward(b)) != cudaSuccess) return e;
      if ((e = backward(b)) != cudaSuccess) return e;
      if ((e = adam_step(lr)) != cudaSuccess) return e;
      if (ep == epochs - 1) {
        double l = 0.0;
        if ((e = cudaMemcpyAsync(&l, loss, sizeof(double), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
        sum += l * b;
        nb += b;
      }
    }
    if (ep == epochs - 1) last = nb ? sum / nb : 0.0;
  }
  // validation: blend = argmin over [0, 1] of |t - blend q|^2 on the held-out rows
  blend = 1.0;
  val_rel = -1.0;
  val_rows.assign(order.begin() + ntr, order.end());
  if (nval > 0) {
    if ((e = cudaMemcpyAsync(idx, order.data() + ntr, sizeof(int) * nval, cudaMemcpyHostToDevice, stream)) !=
        cudaSuccess)
      return e;
    if ((e = cudaMemsetAsync(loss, 0, sizeof(double) * 4, stream)) != cudaSuccess) return e;
    for (int s0 = 0; s0 < nval; s0 += kMaxBatch) {
      const int b = std::min(kMaxBatch, nval - s0);
      k_gather<<<blocks_for((int64_t)b * (din + nf)), 256, 0, stream>>>(xs, ys, idx + s0, b, din, nkin, nf, mu_x, sd_x,
                                                                         mu_y, sd_y, act[0], ybatch);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      if ((e = forward(b)) != cudaSuccess) return e;
      k_val_sums<<<1, 256, 0, stream>>>(ybatch, act[nl], mu_y, sd_y, b, nf, loss + 1);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    double sums[3];
    if ((e = cudaMemcpyAsync(sums, loss + 1, sizeof(sums), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
    blend = sums[1] > 0.0 ? std::min(1.0, std::max(0.0, sums[0] / sums[1])) : 0.0;
    // held-out error of the blended correction relative to plain extrapolation's (correction 0)
    val_rel = sums[2] > 0.0 ? (sums[2] - 2.0 * blend * sums[0] + blend * blend * sums[1]) / sums[2] : 0.0;
  }
  if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
  trained = true;
  if (final_loss) *final_loss = last;
  return cudaSuccess;
}

cudaError_t Mlp::heldout(double* q, double* t, int max_rows, int* rows) {
  const int din = dims[0], nf = dims[nl];
  const int nkin = din - 2 * nf;
  const int n = std::min<int>(max_rows, (int)val_rows.size());
  *rows = n;
  if (n == 0) return cudaSuccess;
  const int* first = val_rows.data() + val_rows.size() - n;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(idx, first, sizeof(int) * n, cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
  for (int s0 = 0; s0 < n; s0 += kMaxBatch) {
    const int b = std::min(kMaxBatch, n - s0);
    k_gather<<<blocks_for((int64_t)b * (din + nf)), 256, 0, stream>>>(xs, ys, idx + s0, b, din, nkin, nf, mu_x, sd_x,
                                                                       mu_y, sd_y, act[0], ybatch);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = forward(b)) != cudaSuccess) return e;
    k_denorm<<<blocks_for((int64_t)b * nf), 256, 0, stream>>>(ybatch, act[nl], mu_y, sd_y, b, nf,
                                                                q + (int64_t)s0 * nf, t + (int64_t)s0 * nf);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t Mlp::gradients(int b, const float* x_host, const float* y_host, float* grad_host, double* loss_host) {
  if (b < 1 || b > kMaxBatch) return cudaErrorInvalidValue;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(act[0], x_host, sizeof(float) * (size_t)b * dims[0], cudaMemcpyHostToDevice, stream)) !=
      cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(ybatch, y_host, sizeof(float) * (size_t)b * dims[nl], cudaMemcpyHostToDevice, stream)) !=
      cudaSuccess)
    return e;
  if ((e = forward(b)) != cudaSuccess) return e;
  if ((e = backward(b)) != cudaSuccess) return e;
  if (grad_host && (e = cudaMemcpyAsync(grad_host, grad, sizeof(float) * nparam, cudaMemcpyDeviceToHost, stream)) !=
                       cudaSuccess)
    return e;
  double l = 0.0;
  if ((e = cudaMemcpyAsync(&l, loss, sizeof(double), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
  if (loss_host) *loss_host = l;
  return cudaSuccess;
}

}  // namespace learn
}  // namespace ib
