// Learned warm start for the moving-body Schur CG: a small multilayer perceptron trained on
// the force histories the solver generates, with hand-written inference and training kernels.
//
//   features x = [kinematics of every body (r0x, r0y, v0x, v0y, theta, Omega), F_{n-1}, F_{n-2}]
//   target   y = F_n - (2 F_{n-1} - F_{n-2})        (the correction to linear extrapolation)
//   network  x~ = (x - mu_x) / sd_x -> tanh(W1 x~ + b1) -> ... -> W_L h + b_L = y~,
//            y = y~ * sd_y + mu_y,  warm start F_n ~ 2 F_{n-1} - F_{n-2} + y
// Weights are stored BF16 for the products, with FP32 master copies updated by Adam; the
// products run on the tensor cores (tcgen05, FP32 activations as three BF16 parts, FP32
// accumulation in tensor memory).  Reductions (bias gradients, loss, statistics) run in a
// fixed order, so training is reproducible.
#include "ib_common.cuh"
#include "mlp.cuh"
#include "tcgen05.cuh"

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

using namespace tc;

template <typename T> __device__ __forceinline__ float ldf(const T* p, int64_t i);
template <> __device__ __forceinline__ float ldf<float>(const float* p, int64_t i) { return p[i]; }
template <> __device__ __forceinline__ float ldf<__nv_bfloat16>(const __nv_bfloat16* p, int64_t i) {
  return __bfloat162float(p[i]);
}

enum Epi : int { kStore = 0, kBias = 1, kBiasTanh = 2 };

// The network's products on the tensor cores: C[M x N] = op(A)[M x K] op(B)[K x N] (+ bias[n],
// tanh), with A FP32 stored [M][K] (TA false) or [K][M] (TA true) and B FP32 or BF16 stored
// [K][N] (TB false) or [N][K] (TB true).
//
// FP32 operands are split into three BF16 parts x = x1 + x2 + x3 (each the BF16 rounding of the
// remainder of the previous ones, 24 significant bits together); BF16 operands (the weights) are
// one exact part.  The products x_i y_j with i + j <= 2 (0-based; the dropped ones are below
// 2^-24 of the terms) accumulate in FP32 in tensor memory, so the result has FP32 accuracy: 3
// tcgen05.mma per K step against BF16 weights, 6 between two FP32 operands.
//
// One CTA = 128 rows x 128 columns of C, K in chunks of 64 (one 128-byte swizzle row of BF16):
// the 8 warps load the chunk (coalesced along whichever of the operand's axes is contiguous),
// split it and store the parts in the K-major swizzled layout; one thread issues the MMAs (M 128,
// N 128, K 16) and commits them to an mbarrier that frees the single stage.  The products are
// small (rows = a minibatch, columns = layer widths), so the chunks are not pipelined.  Waits
// are bounded: on expiry the CTA sets the status flag, drains its MMAs (bounded), frees its
// tensor memory and returns.
constexpr int kTM = 128, kTN = 128, kTK = 64, kTThreads = 256;
constexpr int kPart = kTM * kTK * 2;  // bytes of one BF16 part of a 128 x 64 operand tile

template <typename T>
__device__ __forceinline__ void store_parts(unsigned char* base, int nparts, uint32_t off, float a, float b) {
  if (nparts == 1) {
    const uint32_t w = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
                       ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
    *reinterpret_cast<uint32_t*>(base + off) = w;
    return;
  }
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const __nv_bfloat16 ah = __float2bfloat16_rn(a), bh = __float2bfloat16_rn(b);
    *reinterpret_cast<uint32_t*>(base + q * kPart + off) =
        (uint32_t)__bfloat16_as_ushort(ah) | ((uint32_t)__bfloat16_as_ushort(bh) << 16);
    a -= __bfloat162float(ah);
    b -= __bfloat162float(bh);
  }
}

// the 128 x 64 tile (rows r0.., K k0..) of X(r, k) = X[r rs + k ks] into its swizzled parts
template <typename T, bool KCONTIG>
__device__ __forceinline__ void load_tile(const T* __restrict__ X, int64_t rs, int64_t ks, int r0, int R, int k0,
                                          int K, unsigned char* parts, int nparts) {
#pragma unroll 4
  for (int t = 0; t < kTM * (kTK / 2) / kTThreads; ++t) {
    const int i = t * kTThreads + (int)threadIdx.x;
    const int r = KCONTIG ? (i >> 5) : (i & (kTM - 1));
    const int kp = KCONTIG ? (i & 31) : (i >> 7);
    const int gr = r0 + r, k = k0 + 2 * kp;
    float a = 0.f, b = 0.f;
    if (gr < R) {
      if (k < K) a = ldf(X, (int64_t)gr * rs + (int64_t)k * ks);
      if (k + 1 < K) b = ldf(X, (int64_t)gr * rs + (int64_t)(k + 1) * ks);
    }
    store_parts<T>(parts, nparts, sw128_off(r, kp), a, b);
  }
}

template <bool TA, bool TB, typename TBt, int EPI>
__global__ void __launch_bounds__(kTThreads, 1)
k_tcgemm(int M, int N, int K, const float* __restrict__ A, const TBt* __restrict__ B, float* __restrict__ C,
         const float* __restrict__ bias, int* __restrict__ status) {
  constexpr int NPB = std::is_same<TBt, float>::value ? 3 : 1;
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t done;
  __shared__ uint32_t tmem_slot;
  unsigned char* sm = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  unsigned char* pa = sm;                // 3 parts of the A tile
  unsigned char* pb = sm + 3 * kPart;    // NPB parts of the B tile
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
  if (tid == 0) {
    mbar_init(&done, 1);
    fence_mbar_init();
    fence_async_smem();
  }
  if (warp == 0) tmem_alloc(&tmem_slot, kTN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  constexpr uint32_t kIdesc = idesc_bf16_mn<kTM, kTN>();
  int committed = 0, drained = 0;
  bool bad = false;
  const int nkc = (K + kTK - 1) / kTK;
  for (int c = 0; c < nkc; ++c) {
    // A(m, k) = A[m K + k] or A[k M + m];  B(n, k) = B[n K + k] or B[k N + n]
    load_tile<float, !TA>(A, TA ? 1 : K, TA ? M : 1, m0, M, c * kTK, K, pa, 3);
    load_tile<TBt, TB>(B, TB ? K : 1, TB ? 1 : N, n0, N, c * kTK, K, pb, NPB);
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int ks = 0; ks < kTK / 16; ++ks) {
        const uint32_t o32 = ks * 32;  // 16 BF16 = 32 bytes along K inside the swizzle row
        bool first = c == 0 && ks == 0;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < NPB; ++j)
            if (i + j <= 2) {
              umma_bf16(tmem, sw128_desc(smem_u32(pa + i * kPart) + o32), sw128_desc(smem_u32(pb + j * kPart) + o32),
                        kIdesc, first ? 0u : 1u);
              first = false;
            }
      }
      umma_commit(&done);
      ++committed;
      if (!mbar_wait(&done, (uint32_t)c & 1)) bad = true;
      else drained = committed;
    }
    if (__syncthreads_or(bad)) break;
  }
  if (bad) {
    if (tid == 0) {
      atomicExch(status, 1);
      for (int k = drained; k < committed; ++k) mbar_wait(&done, (uint32_t)k & 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTN);
    return;
  }
  tc_fence_after();
  // epilogue: warp w reads TMEM lanes 32 (w & 3) .. + 31 (rows), columns of half w >> 2
  const int q = warp & 3, half = warp >> 2;
  const int m = m0 + 32 * q + lane;
  const uint32_t tb = tmem + ((uint32_t)(32 * q) << 16);
#pragma unroll 1
  for (int cc = 0; cc < kTN / 2; cc += 16) {
    const int col0 = half * (kTN / 2) + cc;
    float v[16];
    tmem_ld16(tb + (uint32_t)col0, v);
    if (m >= M) continue;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int n = n0 + col0 + i;
      if (n >= N) continue;
      float x = v[i];
      if (EPI != kStore) x += bias[n];
      if (EPI == kBiasTanh) x = tanhf(x);
      C[(int64_t)m * N + n] = x;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTN);
}

constexpr int kTSmem = 6 * kPart + 1024;  // 3 + 3 operand parts + alignment slack

template <bool TA, bool TB, typename TBt, int EPI>
cudaError_t gemm_attr() {
  return cudaFuncSetAttribute(k_tcgemm<TA, TB, TBt, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTSmem);
}

template <bool TA, bool TB, typename TBt, int EPI>
cudaError_t gemm(int M, int N, int K, const float* A, const TBt* B, float* C, const float* bias, int* status,
                 cudaStream_t s) {
  dim3 grid((N + kTN - 1) / kTN, (M + kTM - 1) / kTM);
  k_tcgemm<TA, TB, TBt, EPI><<<grid, kTThreads, kTSmem, s>>>(M, N, K, A, B, C, bias, status);
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
cudaError_t Mlp::init(int din_, int dout_, int hidden, int nhidden, int capacity, uint64_t seed, cudaStream_t s,
                      int* status_flag) {
  release();
  stream = s;
  status = status_flag;
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
  // shared-memory limits of the tensor-core products (set outside any stream capture)
  if ((e = gemm_attr<false, true, __nv_bfloat16, kBiasTanh>()) != cudaSuccess ||
      (e = gemm_attr<false, true, __nv_bfloat16, kBias>()) != cudaSuccess ||
      (e = gemm_attr<true, false, float, kStore>()) != cudaSuccess ||
      (e = gemm_attr<false, false, __nv_bfloat16, kStore>()) != cudaSuccess)
    return e;
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
    cudaError_t e = (l + 1 < nl)
                        ? gemm<false, true, __nv_bfloat16, kBiasTanh>(b, N, K, act[l], W, act[l + 1], bias, status, stream)
                        : gemm<false, true, __nv_bfloat16, kBias>(b, N, K, act[l], W, act[l + 1], bias, status, stream);
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
    if ((e = gemm<true, false, float, kStore>(N, K, b, dact[l + 1], act[l], grad + woff[l], nullptr, status, stream)) !=
        cudaSuccess)
      return e;
    k_colsum<<<(N + 127) / 128, 128, 0, stream>>>(dact[l + 1], grad + boff[l], b, N);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // dX = dZ W  [b x K]
    if (l > 0) {
      if ((e = gemm<false, false, __nv_bfloat16, kStore>(b, K, N, dact[l + 1], wbf + woff[l], dact[l], nullptr, status,
                                                         stream)) != cudaSuccess)
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
