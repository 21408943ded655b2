// Line-parallel x passes (see dstw.cuh), kernels and launchers shared by dstw_xf.cu (forward
// pass) and dstw_xi.cu (inverse pass): the first and last pass of every Poisson / CN solve
// on grids whose axes have warp-per-line tables.
//
//   k_wxf: rows of the input -> prologue (load, apply_bc edges, refinement residual) -> S_x
//          -> stored transposed (column by column) for the y pass
//   k_wxi: transposed intermediate -> S_x -> epilogue (store, subtract, add the FP32 base
//          iterate) into row-major output
// A block owns kLines consecutive rows; the transposing copies go through the rows' shared
// buffers so that both the row-major and the column-major side are contiguous in memory.
#pragma once

#include "dstw.cuh"

namespace ib {
namespace {

using wdst::line_lb;
using wdst::kLines;
using wdst::Shape;
using wdst::line_dst;
using wdst::line_sync;

template <typename T, typename Tin, int P, int NL, int PRO, bool kBC>
__global__ void __launch_bounds__(kLines * NL, IB_WDST_XMINB)
k_wxf(Geometry g, DstAxis<T> ax, XArgs a) {
  pdl_begin();
  // exact arithmetic of the prologue: FP64, or float-float when the input is float-float
  using A = typename std::conditional<is_df64<Tin>::value, df64, double>::type;
  using Sh = Shape<T, P, NL>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int w = threadIdx.x / NL, lane = threadIdx.x % NL;
  T* U = sm + w * Sh::kStride;
  T* D = U + Sh::kU;
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const int total = a.batch * nrow;
  const Tin* in = static_cast<const Tin*>(a.in);
  T* out = static_cast<T*>(a.out);
  for (int base = blockIdx.x * kLines; base < total; base += gridDim.x * kLines) {
    const int row = base + w;
    if (row < total) {
      const int b = row / nrow, J = row - b * nrow;
      const int64_t off = (int64_t)b * a.stride + (int64_t)J * ncol;
      const Tin* src = in + off;
      if constexpr ((PRO == kProResid || PRO == kProResidD) && is_df64<Tin>::value) {
        // refinement residual r = b [+ apply_bc] - M x, x = x0 [+ x1] (FP32 parts, or the two
        // parts of a float-float x0), with M x = mc x + ma (4 x - neighbours) to float-float
        // accuracy.  float(r) feeds the FP32 transform; r itself can be kept (resid_out).
        constexpr bool kD = PRO == kProResidD;
        const float* x0 = kD ? nullptr : a.base + off;
        const float* x1 = (!kD && a.base2) ? a.base2 + off : nullptr;
        const df64* xd = kD ? a.based + off : nullptr;
        const double mcd = a.mc[b * a.mstep];
        const df64 mc = df64(mcd), ma = df64(a.ma[b * a.mstep]);
        const A* bc = kBC ? static_cast<const A*>(a.bc) + (int64_t)b * g.nbc : nullptr;
        const bool fac1 = a.bcfac == 1.0;
        const df64 fac = df64(a.bcfac);
        df64* rout = a.resid_out ? static_cast<df64*>(a.resid_out) + off : nullptr;
        const float* xs = (!kD && J > 0) ? x0 - ncol : nullptr;
        const float* xn = (!kD && J < nrow - 1) ? x0 + ncol : nullptr;
        const float* ys = (x1 && J > 0) ? x1 - ncol : nullptr;
        const float* yn = (x1 && J < nrow - 1) ? x1 + ncol : nullptr;
        const df64* ds = (kD && J > 0) ? xd - ncol : nullptr;
        const df64* dn = (kD && J < nrow - 1) ? xd + ncol : nullptr;
        // ring terms of this row: the whole row at the bottom / top edge, one element at the
        // left / right edge, loaded at their use (loading them with a float-float iterate
        // spilled 200 bytes at P = 16 and took 1.155 instead of 1.139 ms per 1024^2 x 4 step)
        const A* bcrow = (kBC && J == 0) ? bc + g.B + 1 : ((kBC && J == nrow - 1) ? bc + g.T + 1 : nullptr);
        // eight elements per lane per round, every load of a round issued before any use
        constexpr int R = 8;
        for (int I0 = lane; I0 < ncol; I0 += NL * R) {
          float c0[R], w0[R], e0[R], s0[R], n0[R];
          float c1[kD ? R : 1], w1[kD ? R : 1], e1[kD ? R : 1], s1[kD ? R : 1], n1[kD ? R : 1];
          df64 v[R];
#pragma unroll
          for (int u = 0; u < R; ++u) {
            const int I = I0 + NL * u;
            const bool ok = I < ncol;
            if constexpr (kD) {
              const df64 z(0.0f);
              const df64 c = ok ? xd[I] : z, ww = (ok && I > 0) ? xd[I - 1] : z, e = (I < ncol - 1) ? xd[I + 1] : z;
              const df64 ss = (ok && ds) ? ds[I] : z, nn = (ok && dn) ? dn[I] : z;
              c0[u] = c.hi; w0[u] = ww.hi; e0[u] = e.hi; s0[u] = ss.hi; n0[u] = nn.hi;
              c1[u] = c.lo; w1[u] = ww.lo; e1[u] = e.lo; s1[u] = ss.lo; n1[u] = nn.lo;
            } else {
              c0[u] = ok ? x0[I] : 0.0f;
              w0[u] = (ok && I > 0) ? x0[I - 1] : 0.0f;
              e0[u] = (I < ncol - 1) ? x0[I + 1] : 0.0f;
              s0[u] = (ok && xs) ? xs[I] : 0.0f;
              n0[u] = (ok && xn) ? xn[I] : 0.0f;
            }
            v[u] = ok ? src[I] : df64(0.0f);
          }
          df64 lap[R], xv[R];
#pragma unroll
          for (int u = 0; u < R; ++u) {
            lap[u] = lap5_exact(c0[u], w0[u], e0[u], s0[u], n0[u]);
            xv[u] = df64(c0[u]);
          }
          if constexpr (kD) {
#pragma unroll
            for (int u = 0; u < R; ++u) {
              lap[u] = add_sloppy(lap[u], lap5_exact(c1[u], w1[u], e1[u], s1[u], n1[u]));
              xv[u] = two_sum(c0[u], c1[u]);
            }
          }
          if (x1) {
#pragma unroll
            for (int u = 0; u < R; ++u) {
              const int I = I0 + NL * u;
              const bool ok = I < ncol;
              c0[u] = ok ? x1[I] : 0.0f;
              w0[u] = (ok && I > 0) ? x1[I - 1] : 0.0f;
              e0[u] = (I < ncol - 1) ? x1[I + 1] : 0.0f;
              s0[u] = (ok && ys) ? ys[I] : 0.0f;
              n0[u] = (ok && yn) ? yn[I] : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < R; ++u) {
              lap[u] = add_sloppy(lap[u], lap5_exact(c0[u], w0[u], e0[u], s0[u], n0[u]));
              xv[u] = two_sum(xv[u].hi, c0[u]);
            }
          }
#pragma unroll
          for (int u = 0; u < R; ++u) {
            const int I = I0 + NL * u;
            if (I >= ncol) break;
            df64 mx = ma * lap[u];
            if (mcd == 1.0) mx = add_sloppy(mx, xv[u]);
            else if (mcd != 0.0) mx = add_sloppy(mx, mc * xv[u]);
            df64 vv = v[u];
            if constexpr (kBC) {
              auto addbc = [&](df64 q) { vv = add_sloppy(vv, fac1 ? q : fac * q); };
              if (bcrow) addbc(bcrow[I]);
              if (I == 0) addbc(bc[g.L + 1 + J]);
              if (I == ncol - 1) addbc(bc[g.R + 1 + J]);
            }
            U[I + 1] = (T)((vv.hi - mx.hi) + (vv.lo - mx.lo));
            if (rout) rout[I] = add_sloppy(vv, -mx);
          }
        }
      } else if (PRO == kProLoad && !kBC && std::is_same<Tin, T>::value) {
        constexpr int LB = line_lb<T, P, NL>();
        for (int I0 = lane; I0 < ncol; I0 += LB * NL) {
          T v[LB];
#pragma unroll
          for (int u = 0; u < LB; ++u) v[u] = (I0 + NL * u < ncol) ? (T)src[I0 + NL * u] : T(0);
#pragma unroll
          for (int u = 0; u < LB; ++u)
            if (I0 + NL * u < ncol) U[I0 + NL * u + 1] = v[u];
        }
      } else {
        const A* bc = kBC ? static_cast<const A*>(a.bc) + (int64_t)b * g.nbc : nullptr;
        const A fac = A(a.bcfac);
        const float* x0 = (PRO == kProResid) ? a.base + off : nullptr;
        const float* x1 = (PRO == kProResid && a.base2) ? a.base2 + off : nullptr;
        const A mc = (PRO == kProResid) ? A(a.mc[b * a.mstep]) : A(0.0);
        const A ma = (PRO == kProResid) ? A(a.ma[b * a.mstep]) : A(0.0);
#pragma unroll 4
        for (int I = lane; I < ncol; I += NL) {
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
          U[I + 1] = (T)v;
        }
      }
      line_sync<NL>(w + 1);
      line_dst<T, P, NL>(U, D, ax, lane, w + 1);
    }
    __syncthreads();
    // transposed store: thread (ww = tid mod kLines) copies row base + ww, kLines consecutive
    // threads write the block's rows of one column I next to each other
    {
      const int ww = threadIdx.x & (kLines - 1);
      const int rr = base + ww;
      if (rr < total) {
        const int b = rr / nrow, J = rr - b * nrow;
        T* o = out + (int64_t)b * a.stride + J;
        const T* srow = sm + ww * Sh::kStride + 1;
        constexpr int step = NL;
#pragma unroll 8
        for (int I = threadIdx.x / kLines; I < ncol; I += step) o[(int64_t)I * nrow] = srow[I];
      }
    }
    __syncthreads();
  }
}

template <typename T, typename Tout, int P, int NL, int EPI>
__global__ void __launch_bounds__(kLines * NL, IB_WDST_XMINB)
k_wxi(Geometry g, DstAxis<T> ax, XArgs a) {
  pdl_begin();
  using A = typename std::conditional<is_df64<Tout>::value, df64, double>::type;
  using Sh = Shape<T, P, NL>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int w = threadIdx.x / NL, lane = threadIdx.x % NL;
  T* U = sm + w * Sh::kStride;
  T* D = U + Sh::kU;
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const int total = a.batch * nrow;
  const T* in = static_cast<const T*>(a.in);
  Tout* out = static_cast<Tout*>(a.out);
  for (int base = blockIdx.x * kLines; base < total; base += gridDim.x * kLines) {
    // transposed load (the mirror of k_wxf's store), eight loads in flight per thread
    {
      const int ww = threadIdx.x & (kLines - 1);
      const int rr = base + ww;
      if (rr < total) {
        const int b = rr / nrow, J = rr - b * nrow;
        const T* src = in + (int64_t)b * a.stride + J;
        T* drow = sm + ww * Sh::kStride + 1;
        constexpr int step = NL;
        constexpr int LB = line_lb<T, P, NL>();
        for (int I0 = threadIdx.x / kLines; I0 < ncol; I0 += LB * step) {
          T v[LB];
#pragma unroll
          for (int u = 0; u < LB; ++u) {
            const int I = I0 + u * step;
            v[u] = I < ncol ? src[(int64_t)I * nrow] : T(0);
          }
#pragma unroll
          for (int u = 0; u < LB; ++u) {
            const int I = I0 + u * step;
            if (I < ncol) drow[I] = v[u];
          }
        }
      }
    }
    __syncthreads();
    const int row = base + w;
    if (row < total) {
      const int b = row / nrow, J = row - b * nrow;
      const int64_t off = (int64_t)b * a.stride + (int64_t)J * ncol;
      line_dst<T, P, NL>(U, D, ax, lane, w + 1);
      Tout* dst = out + off;
      if (EPI == kEpiStore) {
#pragma unroll 8
        for (int I = lane; I < ncol; I += NL) dst[I] = (Tout)U[I + 1];
      } else if (EPI == kEpiSub) {
        const A* sf = static_cast<const A*>(a.sub_from) + off;
#pragma unroll 4
        for (int I = lane; I < ncol; I += NL) dst[I] = (Tout)(sf[I] - A(U[I + 1]));
      } else if constexpr (is_df64<Tout>::value) {
        // x = x0 [+ x1] + d: the FP32 parts summed error-free, the (small) correction added
        // to the low part
        const float* bs = a.base ? a.base + off : nullptr;
        const float* bs2 = a.base2 ? a.base2 + off : nullptr;
        constexpr bool kF = EPI == kEpiSubAddBase || EPI == kEpiAddTo;
        const df64* sf = kF ? static_cast<const df64*>(a.sub_from) + off : nullptr;
        df64* s2 = (EPI == kEpiAddTo && a.sub2) ? static_cast<df64*>(a.sub2) + off : nullptr;
        // up to sixteen elements per lane per round on one-warp lines (1.167 vs 1.172 ms per
        // 1024^2 x 4 mixed step with eight; 32 spills), eight on two-warp lines (64 registers)
        constexpr int R = NL == 32 ? (2 * P < 16 ? 2 * P : 16) : 8;
        for (int I0 = lane; I0 < ncol; I0 += NL * R) {
          float b0[R], b1[R];
          df64 f[R];
#pragma unroll
          for (int u = 0; u < R; ++u) {
            const int I = I0 + NL * u;
            const bool ok = I < ncol;
            b0[u] = (ok && bs) ? bs[I] : 0.0f;
            b1[u] = (ok && bs2) ? bs2[I] : 0.0f;
            if (kF) f[u] = ok ? sf[I] : df64(0.0f);
          }
#pragma unroll
          for (int u = 0; u < R; ++u) {
            const int I = I0 + NL * u;
            if (I >= ncol) break;
            const df64 x01 = two_sum(b0[u], b1[u]);
            const df64 xv = two_sum(x01.hi, x01.lo + (float)U[I + 1]);
            const df64 y = (EPI == kEpiSubAddBase) ? add_sloppy(f[u], -xv) : (EPI == kEpiAddTo) ? add_sloppy(f[u], xv) : xv;
            dst[I] = y;
            if (EPI == kEpiAddTo && s2) s2[I] = add_sloppy(s2[I], -y);
          }
        }
      } else {
        const float* bs = a.base + off;
        const float* bs2 = a.base2 ? a.base2 + off : nullptr;
        const A* sf = (EPI == kEpiSubAddBase) ? static_cast<const A*>(a.sub_from) + off : nullptr;
#pragma unroll 4
        for (int I = lane; I < ncol; I += NL) {
          A xv = A(bs[I]);
          if (bs2) xv = xv + A(bs2[I]);
          xv = xv + A(U[I + 1]);
          dst[I] = (Tout)((EPI == kEpiSubAddBase) ? sf[I] - xv : xv);
        }
      }
    }
    __syncthreads();
  }
}

template <typename T, int P, int NL>
size_t smem_bytes() {
  return (size_t)kLines * Shape<T, P, NL>::kStride * sizeof(T);
}

template <typename T, typename Tin, int P, int NL, int PRO, bool kBC>
cudaError_t launch_fwd(const Geometry& g, const DstAxis<T>& ax, const XArgs& a, cudaStream_t s) {
  auto k = k_wxf<T, Tin, P, NL, PRO, kBC>;
  const size_t smem = smem_bytes<T, P, NL>();
  cudaError_t e = set_smem_limit((const void*)k, smem);
  if (e != cudaSuccess) return e;
  const int total = a.batch * (g.ny - 1);
  return launch_k(k, dim3((total + kLines - 1) / kLines), dim3(kLines * NL), smem, s, g, ax, a);
}

template <typename T, typename Tin, int P, int NL>
cudaError_t fwd_p(const Geometry& g, const DstAxis<T>& ax, const XArgs& a, cudaStream_t s) {
  const bool bc = a.bc != nullptr;
  if (a.pro == kProResid) {
    // the refinement residual belongs to the mixed path (float-float input)
    if constexpr (is_df64<Tin>::value) {
      if (!a.base || !a.mc || !a.ma) return cudaErrorInvalidValue;
      return bc ? launch_fwd<T, Tin, P, NL, kProResid, true>(g, ax, a, s)
                : launch_fwd<T, Tin, P, NL, kProResid, false>(g, ax, a, s);
    }
    return cudaErrorInvalidValue;
  }
  if (a.pro == kProResidD) {
    if constexpr (is_df64<Tin>::value) {
      if (!a.based || !a.mc || !a.ma) return cudaErrorInvalidValue;
      return bc ? launch_fwd<T, Tin, P, NL, kProResidD, true>(g, ax, a, s)
                : launch_fwd<T, Tin, P, NL, kProResidD, false>(g, ax, a, s);
    }
    return cudaErrorInvalidValue;
  }
  return bc ? launch_fwd<T, Tin, P, NL, kProLoad, true>(g, ax, a, s) : launch_fwd<T, Tin, P, NL, kProLoad, false>(g, ax, a, s);
}

template <typename T, typename Tout, int P, int NL, int EPI>
cudaError_t launch_inv(const Geometry& g, const DstAxis<T>& ax, const XArgs& a, cudaStream_t s) {
  auto k = k_wxi<T, Tout, P, NL, EPI>;
  const size_t smem = smem_bytes<T, P, NL>();
  cudaError_t e = set_smem_limit((const void*)k, smem);
  if (e != cudaSuccess) return e;
  const int total = a.batch * (g.ny - 1);
  return launch_k(k, dim3((total + kLines - 1) / kLines), dim3(kLines * NL), smem, s, g, ax, a);
}

// epilogues per output type: FP64 path store / subtract; mixed path FP32 store of the iterate
// and float-float sums with the base iterate
template <typename T, typename Tout, int P, int NL>
cudaError_t inv_p(const Geometry& g, const DstAxis<T>& ax, const XArgs& a, cudaStream_t s) {
  if (a.bc) return cudaErrorInvalidValue;
  if constexpr (std::is_same<Tout, T>::value) {
    if (a.epi == kEpiStore) return launch_inv<T, Tout, P, NL, kEpiStore>(g, ax, a, s);
    if constexpr (std::is_same<T, double>::value) {
      if (a.epi == kEpiSub) return launch_inv<T, Tout, P, NL, kEpiSub>(g, ax, a, s);
    }
    return cudaErrorInvalidValue;
  } else {
    // a float-float result needs no base (a transform-only solve); a double one does
    if (!a.base && (a.base2 || !is_df64<Tout>::value)) return cudaErrorInvalidValue;
    if (a.epi == kEpiAddBase) return launch_inv<T, Tout, P, NL, kEpiAddBase>(g, ax, a, s);
    if (a.epi == kEpiSubAddBase) return launch_inv<T, Tout, P, NL, kEpiSubAddBase>(g, ax, a, s);
    if constexpr (is_df64<Tout>::value) {
      if (a.epi == kEpiAddTo) return launch_inv<T, Tout, P, NL, kEpiAddTo>(g, ax, a, s);
    }
    return cudaErrorInvalidValue;
  }
}

}  // namespace
}  // namespace ib
