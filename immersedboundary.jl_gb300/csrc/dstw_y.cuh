// Warp-per-line y pass (see dstw.cuh): one warp per column of the transposed intermediate,
// which is contiguous in memory: S_y, spectral multiply (per-slot multipliers, column-major
// in spectral space) and S_y again, in place.  Compiled for two occupancies (MINB resident
// blocks per SM: dstw_y.cu MINB = IB_WDST_YMINB, dstw_y8.cu MINB = 8); the axis' wMinB, which
// the setup-time autotuner may change, picks one.
#pragma once

#include "dstw.cuh"

namespace ib {
namespace {

using wdst::line_lb;
using wdst::kLines;
using wdst::Shape;
using wdst::line_dst;
using wdst::line_sync;

template <typename T, int P, int NL, SpecOp OP, int MINB>
__global__ void __launch_bounds__(kLines * NL, MINB)
k_wy(Geometry g, DstAxis<T> ax, YPassArgs<T> a) {
  pdl_begin();
  using Sh = Shape<T, P, NL>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = threadIdx.x / NL, lane = threadIdx.x % NL;
  T* U = reinterpret_cast<T*>(smem_raw) + w * Sh::kStride;
  T* D = U + Sh::kU;
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const int total = a.batch * ncol;
  // the whole line in one or two round trips per lane (fewer registers at 8 blocks per SM)
  constexpr int LB = MINB >= 8 && line_lb<T, P, NL>() > 16 ? 16 : line_lb<T, P, NL>();
  for (int col = blockIdx.x * kLines + w; col < total; col += gridDim.x * kLines) {
    const int b = col / ncol, I = col - b * ncol;
    const int64_t off = (int64_t)b * a.stride + (int64_t)I * nrow;
    const T* src = a.in1 + off;
    for (int J0 = lane; J0 < nrow; J0 += LB * NL) {
      T v[LB];
#pragma unroll
      for (int u = 0; u < LB; ++u) v[u] = (J0 + NL * u < nrow) ? src[J0 + NL * u] : T(0);
#pragma unroll
      for (int u = 0; u < LB; ++u)
        if (J0 + NL * u < nrow) U[J0 + NL * u + 1] = v[u];
    }
    line_sync<NL>(w + 1);
    line_dst<T, P, NL>(U, D, ax, lane, w + 1);
    if (OP == SpecOp::kScale) {
      const T* m = a.m1 + (int64_t)b * a.mstride + (int64_t)I * nrow;
      for (int J0 = lane; J0 < nrow; J0 += LB * NL) {
        T v[LB];
#pragma unroll
        for (int u = 0; u < LB; ++u) v[u] = (J0 + NL * u < nrow) ? __ldg(&m[J0 + NL * u]) : T(0);
#pragma unroll
        for (int u = 0; u < LB; ++u)
          if (J0 + NL * u < nrow) U[J0 + NL * u + 1] *= v[u];
      }
      line_sync<NL>(w + 1);
      line_dst<T, P, NL>(U, D, ax, lane, w + 1);
    } else {
#pragma unroll 8
      for (int J = lane; J < nrow; J += NL) U[J + 1] *= a.scal;
      line_sync<NL>(w + 1);
    }
    T* dst = a.out + off;
#pragma unroll 8
    for (int J = lane; J < nrow; J += NL) dst[J] = U[J + 1];
    line_sync<NL>(w + 1);
  }
}

template <typename T, int P, int NL, int MINB>
cudaError_t launch(const Geometry& g, const DstAxis<T>& ax, const YPassArgs<T>& a, cudaStream_t s) {
  const size_t smem = (size_t)kLines * Shape<T, P, NL>::kStride * sizeof(T);
  const int total = a.batch * (g.nx - 1);
  const int blocks = (total + kLines - 1) / kLines;
  cudaError_t e;
  if (a.op == SpecOp::kFwd) {
    auto k = k_wy<T, P, NL, SpecOp::kFwd, MINB>;
    if ((e = set_smem_limit((const void*)k, smem)) != cudaSuccess) return e;
    if ((e = launch_k(k, dim3(blocks), dim3(kLines * NL), smem, s, g, ax, a)) != cudaSuccess) return e;
  } else {
    auto k = k_wy<T, P, NL, SpecOp::kScale, MINB>;
    if ((e = set_smem_limit((const void*)k, smem)) != cudaSuccess) return e;
    if ((e = launch_k(k, dim3(blocks), dim3(kLines * NL), smem, s, g, ax, a)) != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace

template <typename T, int MINB>
cudaError_t wypass_minb(const Geometry& g, const DstAxis<T>& ax, const YPassArgs<T>& a, cudaStream_t s) {
  switch (ax.wNL * 100 + ax.wP) {
#define IB_WCASE(NL, P) \
  case NL * 100 + P: return launch<T, P, NL, MINB>(g, ax, a, s);
    IB_WDST_COMBOS(IB_WCASE)
#undef IB_WCASE
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace ib
