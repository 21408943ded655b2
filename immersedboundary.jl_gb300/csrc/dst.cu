// Batched 2-D DST-I passes: the Poisson / Crank-Nicolson solves of the IBPM step.
//
// Replaces the FFTW RODFT00 plan + `LaplacianInv` call of the reference
// (src/streamfcn/fluid-ops.jl:19-56) and the CN multipliers of `A_Ainv_linearmaps`
// (src/streamfcn/cnab/ops.jl:14-42).
//
// A group of kGroup = 64 threads transforms one line (a row for the x pass, a column for the
// y pass) held in shared memory.  The DST-I of the n-1 interior values of an n-cell axis,
//     F_k = sum_{j=1}^{n-1} y_j sin(pi j k / n),
// is computed without the 2x padding of an odd extension:
//   1. u_j = sin(pi j/n)(y_j + y_{n-j}) + (y_j - y_{n-j})/2         (in place, pairs j, n-j)
//   2. U = real DFT_n(u) through a complex Stockham FFT of length M = n/2
//      (mixed radix 8/4/2/3/5, ping-pong buffers padded one slot in nine against bank
//      conflicts, twiddles from a table)
//   3. split: F_{2k} = -Im U_k,  D_k = Re U_k                         (pairs k, M-k)
//   4. F_{2k+1} = D_0/2 + D_1 + ... + D_k                             (prefix sum: per-thread
//      Kahan-compensated chunks, then a scan of the chunk totals across the group)
// (the half-length sine transform of Numerical Recipes "sinft", restated for a warp).
// F is half of FFTW's RODFT00 output; the factor 2 per axis is folded into the
// spectral multipliers, which are multiplied by 16 (exact in binary floating point).
#include "ib_common.cuh"
#include "fft_small.cuh"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

namespace ib {

namespace {

constexpr unsigned kFull = 0xffffffffu;

constexpr int kGroup = 64;  // threads per line

// padded complex index: one spare slot after every 8 complex values
__device__ __forceinline__ int cpad(int i) { return i + (i >> 3); }
// padded index of the prefix-sum workspace: one spare slot after every 32 values
__device__ __forceinline__ int spad(int i) { return i + (i >> 5); }

// One Stockham stage of radix R on a length-M complex line, executed by the kGroup threads of a
// line, from `src` to `dst`.  Butterfly j reads src[j + r*M/R], applies e^{-2 pi i r k/(Ns R)}
// (k = j mod Ns) and writes dst[(j-k)R + k + r Ns].  Buffers use the padded layout, except a
// first stage, which reads the pre-processed line in its natural layout.
template <typename T, int R>
__device__ __forceinline__ void fft_stage(const c2_t<T>* __restrict__ src, c2_t<T>* __restrict__ dst, int M, int Ns,
                                          const c2_t<T>* __restrict__ tw, int t, bool first) {
  using V = c2_t<T>;
  const int nb = M / R;
  const int tstride = M / (Ns * R);
  const bool pow2 = (Ns & (Ns - 1)) == 0;
  for (int j = t; j < nb; j += kGroup) {
    const int k = pow2 ? (j & (Ns - 1)) : (j % Ns);
    V v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = first ? src[j + r * nb] : src[cpad(j + r * nb)];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(&tw[r * k * tstride]));
    }
    Dft<T, R>::run(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[cpad(base + r * Ns)] = v[r];
  }
}

// Shared-memory values per line buffer: the padded complex FFT layout of n reals, rounded to a
// multiple of 4 values so consecutive buffers stay 16-byte aligned.
__host__ __device__ inline int line_buffer_values(int n) { return (n + n / 8 + 8 + 3) & ~3; }
// Prefix-sum workspace: M = n/2 values padded one in 32, plus two exchange slots.
__host__ __device__ inline int scan_buffer_values(int n) { return ((n / 2 + n / 64 + 4) + 3) & ~3; }
// All shared memory of one line.
__host__ __device__ inline int line_values(int n) { return 2 * line_buffer_values(n) + scan_buffer_values(n); }

// In-place DST-I (F convention, see file header) of s[1..n-1] by the kGroup threads of a line
// (t = thread index in the group).  s and scratch hold line_buffer_values(n) values each, D
// holds scan_buffer_values(n); all 16-byte aligned.  Every thread of the block must call it
// (it contains __syncthreads).
template <typename T>
__device__ void dst1_line(T* s, T* scratch, T* D, const DstAxis<T>& ax, int t) {
  using V = c2_t<T>;
  const int n = ax.n, M = ax.M, hn = n >> 1, hM = M >> 1;
  // 1. pre-processing, natural layout
  for (int j = 1 + t; j < hn; j += kGroup) {
    const T a = s[j], b = s[n - j];
    const T sm = a + b, df = T(0.5) * (a - b);
    const T sn = __ldg(&ax.sintab[j]);
    s[j] = fmaT(sn, sm, df);
    s[n - j] = fmaT(sn, sm, -df);
  }
  if (t == 0) {
    s[0] = T(0);
    s[hn] = T(2) * s[hn];
  }
  __syncthreads();
  // 2. complex FFT of length M, ping-pong between s and scratch
  V* src = reinterpret_cast<V*>(s);
  V* dst = reinterpret_cast<V*>(scratch);
  int Ns = 1;
  for (int st = 0; st < ax.nstages; ++st) {
    const int R = ax.radix[st];
    const bool first = st == 0;
    switch (R) {
      case 8: fft_stage<T, 8>(src, dst, M, Ns, ax.tw, t, first); break;
      case 4: fft_stage<T, 4>(src, dst, M, Ns, ax.tw, t, first); break;
      case 2: fft_stage<T, 2>(src, dst, M, Ns, ax.tw, t, first); break;
      case 3: fft_stage<T, 3>(src, dst, M, Ns, ax.tw, t, first); break;
      default: fft_stage<T, 5>(src, dst, M, Ns, ax.tw, t, first); break;
    }
    __syncthreads();
    Ns *= R;
    V* tmp = src;
    src = dst;
    dst = tmp;
  }
  // 3. split the real DFT: pairs (k, M-k) read from the FFT result (padded); F_{2k} goes to
  //    whichever line buffer does not hold the result (natural layout), D_k to the prefix-sum
  //    workspace D
  const V* z = src;
  T* fb = (reinterpret_cast<const T*>(z) == s) ? scratch : s;
  for (int k = 1 + t; k < hM; k += kGroup) {
    const V zk = z[cpad(k)], zm = z[cpad(M - k)];
    const T er = T(0.5) * (zk.x + zm.x), ei = T(0.5) * (zk.y - zm.y);
    const T orr = T(0.5) * (zk.y + zm.y), oi = T(0.5) * (zm.x - zk.x);
    const V w = __ldg(&ax.post[k]);
    const T tr = w.x * orr - w.y * oi, ti = w.x * oi + w.y * orr;
    fb[2 * k] = -(ei + ti);
    D[spad(k)] = er + tr;
    fb[2 * (M - k)] = ei - ti;
    D[spad(M - k)] = er - tr;
  }
  if (t == 0) {
    const V z0 = z[cpad(0)], zh = z[cpad(hM)];
    D[spad(0)] = T(0.5) * (z0.x + z0.y);  // D_0 / 2
    fb[2 * hM] = zh.y;                    // F_M
    D[spad(hM)] = zh.x;
  }
  __syncthreads();
  // 4. F_{2k+1} = sum_{k' <= k} D_k': compensated chunk sums, scan of chunk totals
  const int C = (M + kGroup - 1) / kGroup;
  const int k0 = t * C, k1 = min(M, k0 + C);
  T acc = T(0), comp = T(0);
  for (int k = k0; k < k1; ++k) {
    const T y = D[spad(k)] - comp;
    const T tmp = acc + y;
    comp = (tmp - acc) - y;
    acc = tmp;
    D[spad(k)] = acc;
  }
  // inclusive scan of the chunk totals over the group (two warps)
  const int lane = t & 31, wg = t >> 5;
  T incl = acc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T v = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += v;
  }
  T excl = __shfl_up_sync(kFull, incl, 1);
  if (lane == 0) excl = T(0);
  // warp 1 of the group adds warp 0's total (exchanged through the padding slot after the
  // workspace, which no index above touches)
  T* wtot = D + spad(M) + 1;
  if (wg == 0 && lane == 31) wtot[0] = incl;
  __syncthreads();
  if (wg == 1) excl += wtot[0];
  for (int k = k0; k < k1; ++k) D[spad(k)] += excl;
  __syncthreads();
  if (fb != s) {
    for (int k = t; k < M; k += kGroup) {
      s[2 * k] = fb[2 * k];
      s[2 * k + 1] = D[spad(k)];
    }
  } else {
    for (int k = t; k < M; k += kGroup) s[2 * k + 1] = D[spad(k)];
  }
  if (t == 0) s[0] = T(0);
  __syncthreads();
}

// ------------------------------------------------------------------------------------------
// x pass: kXLines rows per block, kGroup threads per row; see XArgs for the prologue /
// epilogue variants.  Shared memory per row: the line and the FFT scratch.
// ------------------------------------------------------------------------------------------
constexpr int kXLines = 4;

template <typename T, typename Tin, typename Tout, int PRO, int EPI, bool kBC>
__global__ void __launch_bounds__(kXLines * kGroup)
k_xpass(Geometry g, DstAxis<T> ax, XArgs a) {
  // exact arithmetic of the prologue / epilogue: FP64 in the FP64 path, float-float when the
  // pass reads or writes float-float state (mixed path)
  using A = typename std::conditional<is_df64<Tin>::value || is_df64<Tout>::value, df64, double>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int grp = threadIdx.x / kGroup, t = threadIdx.x % kGroup;
  const int lb = line_buffer_values(ax.n);
  T* s = reinterpret_cast<T*>(smem_raw) + grp * line_values(ax.n);
  T* scratch = s + lb;
  T* D = scratch + lb;
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const int total = a.batch * nrow;
  const Tin* in = static_cast<const Tin*>(a.in);
  Tout* out = static_cast<Tout*>(a.out);
  for (int base = blockIdx.x * kXLines; base < total; base += gridDim.x * kXLines) {
    const int row = base + grp;
    const bool active = row < total;
    const int b = active ? row / nrow : 0, J = active ? row - b * nrow : 0;
    const int64_t off = (int64_t)b * a.stride + (int64_t)J * ncol;
    if (active) {
      const Tin* src = in + off;
      if (PRO == kProLoad && !kBC && std::is_same<Tin, T>::value) {
        for (int I = t; I < ncol; I += kGroup) s[I + 1] = (T)src[I];
      } else {
        // input, apply_bc edges (rows then columns, as the reference) and, for the
        // refinement, the residual of the first solution, in exact arithmetic
        const A* bc = kBC ? static_cast<const A*>(a.bc) + (int64_t)b * g.nbc : nullptr;
        const A fac = A(a.bcfac);
        const float* x0 = (PRO == kProResid) ? a.base + off : nullptr;
        const float* x1 = (PRO == kProResid && a.base2) ? a.base2 + off : nullptr;
        const A mc = (PRO == kProResid) ? A(a.mc[b * a.mstep]) : A(0.0);
        const A ma = (PRO == kProResid) ? A(a.ma[b * a.mstep]) : A(0.0);
        for (int I = t; I < ncol; I += kGroup) {
          A v = A(src[I]);
          if (kBC) {
            if (J == 0) v = v + fac * bc[g.B + 1 + I];
            if (J == nrow - 1) v = v + fac * bc[g.T + 1 + I];
            if (I == 0) v = v + fac * bc[g.L + 1 + J];
            if (I == ncol - 1) v = v + fac * bc[g.R + 1 + J];
          }
          if (PRO == kProResid) {
            auto X = [&](int i) { return x1 ? A(x0[i]) + A(x1[i]) : A(x0[i]); };
            const A xc = X(I);
            A lap = A(4.0) * xc;
            if (I > 0) lap = lap - X(I - 1);
            if (I < ncol - 1) lap = lap - X(I + 1);
            if (J > 0) lap = lap - X(I - ncol);
            if (J < nrow - 1) lap = lap - X(I + ncol);
            v = v - (mc * xc + ma * lap);
          }
          s[I + 1] = (T)v;
        }
      }
    }
    __syncthreads();
    dst1_line<T>(s, scratch, D, ax, t);
    if (active) {
      Tout* dst = out + off;
      if (EPI == kEpiStore) {
        for (int I = t; I < ncol; I += kGroup) dst[I] = (Tout)s[I + 1];
      } else if (EPI == kEpiSub) {
        const A* sf = static_cast<const A*>(a.sub_from) + off;
        for (int I = t; I < ncol; I += kGroup) dst[I] = (Tout)(sf[I] - A(s[I + 1]));
      } else {
        const float* bs = a.base + off;
        const float* bs2 = a.base2 ? a.base2 + off : nullptr;
        const A* sf = (EPI == kEpiSubAddBase) ? static_cast<const A*>(a.sub_from) + off : nullptr;
        for (int I = t; I < ncol; I += kGroup) {
          A xv = A(bs[I]);
          if (bs2) xv = xv + A(bs2[I]);
          xv = xv + A(s[I + 1]);
          dst[I] = (Tout)((EPI == kEpiSubAddBase) ? sf[I] - xv : xv);
        }
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------------
// y pass: one block per strip of W columns, kGroup threads per column; forward DST, spectral
// multiply, second DST.  Multipliers are stored column-major in spectral space
// (index I*(ny-1) + J) so a column reads them contiguously.
// Shared memory per column: the line and the FFT scratch.
// ------------------------------------------------------------------------------------------
template <typename T, SpecOp OP>
__global__ void __launch_bounds__(512)
k_ypass(Geometry g, DstAxis<T> ax, YPassArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int W = blockDim.x / kGroup;
  const int grp = threadIdx.x / kGroup, t = threadIdx.x % kGroup;
  const int lb = line_buffer_values(ax.n), lv = line_values(ax.n);
  T* p = reinterpret_cast<T*>(smem_raw) + grp * lv;
  T* sc = p + lb;
  T* D = sc + lb;
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const int nstrips = (ncol + W - 1) / W;
  for (int blk = blockIdx.x; blk < a.batch * nstrips; blk += gridDim.x) {
    const int b = blk / nstrips, I0 = (blk - b * nstrips) * W;
    const int64_t off = (int64_t)b * a.stride;
    T* P = reinterpret_cast<T*>(smem_raw);
    for (int idx = threadIdx.x; idx < nrow * W; idx += blockDim.x) {
      const int J = idx / W, w = idx - J * W, I = I0 + w;
      P[w * lv + J + 1] = (I < ncol) ? a.in1[off + (int64_t)J * ncol + I] : T(0);
    }
    __syncthreads();
    const int I = I0 + grp;
    dst1_line<T>(p, sc, D, ax, t);
    const int64_t mo = (int64_t)b * a.mstride + (int64_t)min(I, ncol - 1) * nrow;
    if (OP == SpecOp::kScale) {
      for (int J = t; J < nrow; J += kGroup) p[J + 1] *= __ldg(&a.m1[mo + J]);
    } else {
      for (int J = t; J < nrow; J += kGroup) p[J + 1] *= a.scal;
    }
    __syncthreads();
    if (OP != SpecOp::kFwd) dst1_line<T>(p, sc, D, ax, t);
    for (int idx = threadIdx.x; idx < nrow * W; idx += blockDim.x) {
      const int J = idx / W, w = idx - J * W, Ic = I0 + w;
      if (Ic < ncol) a.out[off + (int64_t)J * ncol + Ic] = P[w * lv + J + 1];
    }
    __syncthreads();
  }
}

// Raise a kernel's dynamic shared-memory limit once per device (never inside stream capture:
// the first launch of every variant happens while a handle is being created).
cudaError_t ensure_smem(const void* fn, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_pair(fn, dev);
  auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done[key] = bytes;
  return e;
}

// Radix plan of an M-point FFT: powers of two first (8s, then a 4/4, 4 or 2 remainder), then 3s,
// then 5s, so the leading stages have power-of-two strides (k = j & (Ns-1)).
int plan_radices(int M, int* radix) {
  int m = M, ns = 0, p2 = 0, n3 = 0, n5 = 0;
  while (m % 5 == 0) { ++n5; m /= 5; }
  while (m % 3 == 0) { ++n3; m /= 3; }
  while (m % 2 == 0) { ++p2; m /= 2; }
  if (m != 1) return -1;
  int a = p2 / 3, rem = p2 % 3;
  if (rem == 1 && a >= 1) { a -= 1; radix[ns++] = 4; radix[ns++] = 4; }
  else if (rem == 1) { radix[ns++] = 2; }
  else if (rem == 2) { radix[ns++] = 4; }
  for (int i = 0; i < a; ++i) radix[ns++] = 8;
  for (int i = 0; i < n3; ++i) radix[ns++] = 3;
  for (int i = 0; i < n5; ++i) radix[ns++] = 5;
  if (ns > kMaxStages) return -1;
  return ns;
}

template <typename T, typename Tin, typename Tout, int PRO, int EPI, bool kBC>
cudaError_t launch_x1(const Geometry& g, const DstAxis<T>& ax, const XArgs& a, cudaStream_t s) {
  const int total = a.batch * (g.ny - 1);
  const int blocks = (total + kXLines - 1) / kXLines;
  const size_t smem = (size_t)kXLines * line_values(ax.n) * sizeof(T);
  auto k = k_xpass<T, Tin, Tout, PRO, EPI, kBC>;
  cudaError_t e = ensure_smem((const void*)k, smem);
  if (e != cudaSuccess) return e;
  k<<<blocks, kXLines * kGroup, smem, s>>>(g, ax, a);
  return cudaGetLastError();
}

template <typename T, typename Tin, typename Tout, int PRO>
cudaError_t launch_x_epi(const Geometry& g, const DstAxis<T>& ax, const XArgs& a, cudaStream_t s) {
  const bool bc = a.bc != nullptr;
  switch (a.epi) {
    case kEpiStore:
      return bc ? launch_x1<T, Tin, Tout, PRO, kEpiStore, true>(g, ax, a, s)
                : launch_x1<T, Tin, Tout, PRO, kEpiStore, false>(g, ax, a, s);
    case kEpiSub:
      if (bc) return cudaErrorInvalidValue;
      return launch_x1<T, Tin, Tout, PRO, kEpiSub, false>(g, ax, a, s);
    case kEpiAddBase:
      if (bc) return cudaErrorInvalidValue;
      return launch_x1<T, Tin, Tout, PRO, kEpiAddBase, false>(g, ax, a, s);
    case kEpiSubAddBase:
      if (bc) return cudaErrorInvalidValue;
      return launch_x1<T, Tin, Tout, PRO, kEpiSubAddBase, false>(g, ax, a, s);
    default:
      return cudaErrorInvalidValue;
  }
}

template <typename T>
cudaError_t launch_y(const Geometry& g, const DstAxis<T>& ax, const YPassArgs<T>& a, cudaStream_t s) {
  ProfScope prof(kClassYPass, s);
  const size_t per_col = (size_t)line_values(ax.n) * sizeof(T);
  // 4 columns per block for a single array (more blocks than SMs), 8 for batches
  int W = (a.batch > 1) ? 8 : 4;
  while (W > 1 && (size_t)W * per_col > 200 * 1024) W >>= 1;
  const size_t smem = (size_t)W * per_col;
  const int nstrips = (g.nx - 1 + W - 1) / W;
  const int blocks = a.batch * nstrips;
  cudaError_t e;
  if (a.op == SpecOp::kFwd) {
    auto k = k_ypass<T, SpecOp::kFwd>;
    if ((e = ensure_smem((const void*)k, smem)) != cudaSuccess) return e;
    k<<<blocks, W * kGroup, smem, s>>>(g, ax, a);
  } else {
    auto k = k_ypass<T, SpecOp::kScale>;
    if ((e = ensure_smem((const void*)k, smem)) != cudaSuccess) return e;
    k<<<blocks, W * kGroup, smem, s>>>(g, ax, a);
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t set_smem_limit(const void* fn, size_t bytes) { return ensure_smem(fn, bytes); }

// Warp-per-line transforms need M = n/2 = 32 P with P = 2^k or 3 2^k, P <= 32.
static int warp_p(int n) {
  if (n % 2) return 0;
  const int M = n / 2;
  if (M % 32) return 0;
  const int P = M / 32;
  switch (P) {
    case 1: case 2: case 3: case 4: case 6: case 8: case 12: case 16: case 24: case 32: return P;
    default: return 0;
  }
}

bool wdst_axis_supported(int n) { return dst_axis_supported(n) && warp_p(n) > 0; }

bool dst_axis_supported(int n) {
  if (n < 8 || n % 4 != 0 || n / 2 > 1024) return false;
  int r[kMaxStages];
  return plan_radices(n / 2, r) > 0;
}

template <typename T>
cudaError_t AxisTables<T>::build(int n) {
  release();
  if (!dst_axis_supported(n)) return cudaErrorInvalidValue;
  using V = c2_t<T>;
  const int M = n / 2;
  d.n = n;
  d.M = M;
  d.nstages = plan_radices(M, d.radix);
  std::vector<V> tw(M), post(M / 2 + 1);
  std::vector<T> sn(n / 2 + 1);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int p = 0; p < M; ++p) {
    const long double ang = -2.0L * pi * (long double)p / (long double)M;
    tw[p] = mk<V>((T)cosl(ang), (T)sinl(ang));
  }
  for (int k = 0; k <= M / 2; ++k) {
    const long double ang = -2.0L * pi * (long double)k / (long double)n;
    post[k] = mk<V>((T)cosl(ang), (T)sinl(ang));
  }
  for (int j = 0; j <= n / 2; ++j) sn[j] = (T)sinl(pi * (long double)j / (long double)n);
  // lane-ordered tables of the line-parallel transforms: one warp per line.  Two warps per line
  // (IBGB300_LINE_LANES=64; M = 64 P with P = 2..16 so the cross-lane stage stays inside a
  // warp) halve each lane's work but measured slower on GB300 (1024^2 mixed step 1.53 vs
  // 1.48 ms, 2048^2 6.46 vs 5.75 ms): the pair's named barriers cost more than they save.
  int P = warp_p(n), NL = 32;
  const char* lanes_env = std::getenv("IBGB300_LINE_LANES");
  const bool two_warps = lanes_env && std::strcmp(lanes_env, "64") == 0;
  if (P && two_warps && M % 64 == 0 && (M / 64 == 2 || M / 64 == 4 || M / 64 == 8 || M / 64 == 16)) {
    NL = 64;
    P = M / 64;
  }
  d.wP = P;
  d.wNL = NL;
  d.wMinB = IB_WDST_YMINB;
  const int G = !P ? 1 : (NL % P == 0 ? NL / P : 32);
  int lg = 0;
  while ((1 << lg) < G) ++lg;
  std::vector<V> w1((size_t)P * NL), w2((size_t)P * NL), w3((size_t)(lg > 0 ? lg : 1) * NL), ws((size_t)P * NL);
  auto cis = [&](long double num, long double den) {  // e^{-2 pi i num / den}
    const long double ang = -2.0L * pi * num / den;
    return mk<V>((T)cosl(ang), (T)sinl(ang));
  };
  for (int a = 0; a < P; ++a)
    for (int l = 0; l < NL; ++l) {
      w1[a * NL + l] = cis((long double)(l * a), (long double)M);
      w2[a * NL + l] = cis((long double)((l % G) * a), (long double)NL);
      const int m = l + NL * a;
      ws[a * NL + l] = mk<V>((T)sinl(pi * (long double)(2 * m) / (long double)n),
                             (T)sinl(pi * (long double)(2 * m + 1) / (long double)n));
    }
  for (int s = 0; s < lg; ++s) {
    const int h = G >> (s + 1);
    for (int l = 0; l < NL; ++l) {
      const int j = (l % G) % (2 * h);
      w3[s * NL + l] = j >= h ? cis((long double)(j - h), (long double)(2 * h)) : mk<V>((T)1, (T)0);
    }
  }
  const size_t b_tw = tw.size() * sizeof(V), b_post = post.size() * sizeof(V), b_sn = sn.size() * sizeof(T);
  const size_t b_w = (size_t)P * NL * sizeof(V), b_w3 = w3.size() * sizeof(V);
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t o_post = up(b_tw);
  const size_t o_sn = o_post + up(b_post);
  const size_t o_w1 = o_sn + up(b_sn);
  const size_t o_w2 = o_w1 + up(b_w);
  const size_t o_w3 = o_w2 + up(b_w);
  const size_t o_ws = o_w3 + up(b_w3);
  cudaError_t e = cudaMalloc(&mem, o_ws + up(b_w));
  if (e != cudaSuccess) { mem = nullptr; return e; }
  char* base = (char*)mem;
  if ((e = cudaMemcpy(base, tw.data(), b_tw, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
  if ((e = cudaMemcpy(base + o_post, post.data(), b_post, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
  if ((e = cudaMemcpy(base + o_sn, sn.data(), b_sn, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
  if (P) {
    if ((e = cudaMemcpy(base + o_w1, w1.data(), b_w, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
    if ((e = cudaMemcpy(base + o_w2, w2.data(), b_w, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
    if ((e = cudaMemcpy(base + o_w3, w3.data(), b_w3, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
    if ((e = cudaMemcpy(base + o_ws, ws.data(), b_w, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
  }
  d.tw = (const V*)base;
  d.post = (const V*)(base + o_post);
  d.sintab = (const T*)(base + o_sn);
  d.wtw1 = P ? (const V*)(base + o_w1) : nullptr;
  d.wtw2 = P ? (const V*)(base + o_w2) : nullptr;
  d.wtw3 = P ? (const V*)(base + o_w3) : nullptr;
  d.wsn = P ? (const V*)(base + o_ws) : nullptr;
  return cudaSuccess;
}

template <typename T>
void AxisTables<T>::release() {
  if (mem) cudaFree(mem);
  mem = nullptr;
}

template <typename T, typename Tin, typename Tout>
cudaError_t xpass(const Geometry& g, const DstAxis<T>& ax, const XArgs& a, cudaStream_t s) {
  if (ax.n != g.nx) return cudaErrorInvalidValue;
  if (a.batch <= 0) return cudaSuccess;
  ProfScope prof(kClassXPass, s);
  if (a.pro == kProResid) {
    if (!a.base || !a.mc || !a.ma || a.epi != kEpiStore) return cudaErrorInvalidValue;
    return launch_x_epi<T, Tin, Tout, kProResid>(g, ax, a, s);
  }
  return launch_x_epi<T, Tin, Tout, kProLoad>(g, ax, a, s);
}

template <typename T>
cudaError_t ypass(const Geometry& g, const DstAxis<T>& ax, const YPassArgs<T>& a, cudaStream_t s) {
  if (ax.n != g.ny) return cudaErrorInvalidValue;
  if (a.batch <= 0) return cudaSuccess;
  return launch_y<T>(g, ax, a, s);
}

template struct AxisTables<double>;
template struct AxisTables<float>;
// FP64 path: double in, double out.  Mixed path: FP32 transforms fed from float-float inputs,
// FP32 intermediates, float-float results.
template cudaError_t xpass<double, double, double>(const Geometry&, const DstAxis<double>&, const XArgs&, cudaStream_t);
template cudaError_t xpass<float, df64, float>(const Geometry&, const DstAxis<float>&, const XArgs&, cudaStream_t);
template cudaError_t xpass<float, float, float>(const Geometry&, const DstAxis<float>&, const XArgs&, cudaStream_t);
template cudaError_t xpass<float, float, df64>(const Geometry&, const DstAxis<float>&, const XArgs&, cudaStream_t);
template cudaError_t ypass<double>(const Geometry&, const DstAxis<double>&, const YPassArgs<double>&, cudaStream_t);
template cudaError_t ypass<float>(const Geometry&, const DstAxis<float>&, const YPassArgs<float>&, cudaStream_t);


}  // namespace ib
