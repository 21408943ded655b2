// Warp-per-line y pass (see dstw.cuh): one warp per column of the transposed intermediate,
// which is contiguous in memory: S_y, spectral multiply (per-slot multipliers, column-major
// in spectral space) and S_y again, in place.
#include "dstw.cuh"

namespace ib {
namespace {

using wdst::kWarps;
using wdst::Shape;
using wdst::warp_dst;

template <typename T, int P, SpecOp OP>
__global__ void __launch_bounds__(kWarps * 32)
k_wy(Geometry g, DstAxis<T> ax, YPassArgs<T> a) {
  using Sh = Shape<T, P>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* U = reinterpret_cast<T*>(smem_raw) + w * Sh::kStride;
  T* D = U + Sh::kU;
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const int total = a.batch * ncol;
  for (int col = blockIdx.x * kWarps + w; col < total; col += gridDim.x * kWarps) {
    const int b = col / ncol, I = col - b * ncol;
    const int64_t off = (int64_t)b * a.stride + (int64_t)I * nrow;
    const T* src = a.in1 + off;
    for (int J0 = lane; J0 < nrow; J0 += 8 * 32) {
      T v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = (J0 + 32 * u < nrow) ? src[J0 + 32 * u] : T(0);
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (J0 + 32 * u < nrow) U[J0 + 32 * u + 1] = v[u];
    }
    __syncwarp();
    warp_dst<T, P>(U, D, ax, lane);
    if (OP == SpecOp::kScale) {
      const T* m = a.m1 + (int64_t)b * a.mstride + (int64_t)I * nrow;
      for (int J0 = lane; J0 < nrow; J0 += 8 * 32) {
        T v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = (J0 + 32 * u < nrow) ? __ldg(&m[J0 + 32 * u]) : T(0);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (J0 + 32 * u < nrow) U[J0 + 32 * u + 1] *= v[u];
      }
      __syncwarp();
      warp_dst<T, P>(U, D, ax, lane);
    } else {
#pragma unroll 8
      for (int J = lane; J < nrow; J += 32) U[J + 1] *= a.scal;
      __syncwarp();
    }
    T* dst = a.out + off;
#pragma unroll 8
    for (int J = lane; J < nrow; J += 32) dst[J] = U[J + 1];
    __syncwarp();
  }
}

template <typename T, int P>
cudaError_t launch(const Geometry& g, const DstAxis<T>& ax, const YPassArgs<T>& a, cudaStream_t s) {
  const size_t smem = (size_t)kWarps * Shape<T, P>::kStride * sizeof(T);
  const int total = a.batch * (g.nx - 1);
  const int blocks = (total + kWarps - 1) / kWarps;
  cudaError_t e;
  if (a.op == SpecOp::kFwd) {
    auto k = k_wy<T, P, SpecOp::kFwd>;
    if ((e = set_smem_limit((const void*)k, smem)) != cudaSuccess) return e;
    k<<<blocks, kWarps * 32, smem, s>>>(g, ax, a);
  } else {
    auto k = k_wy<T, P, SpecOp::kScale>;
    if ((e = set_smem_limit((const void*)k, smem)) != cudaSuccess) return e;
    k<<<blocks, kWarps * 32, smem, s>>>(g, ax, a);
  }
  return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t wypass(const Geometry& g, const DstAxis<T>& ax, const YPassArgs<T>& a, cudaStream_t s) {
  if (ax.n != g.ny || !ax.wP) return cudaErrorInvalidValue;
  if (a.batch <= 0) return cudaSuccess;
  ProfScope prof(kClassYPass, s);
  switch (ax.wP) {
    case 1: return launch<T, 1>(g, ax, a, s);
    case 2: return launch<T, 2>(g, ax, a, s);
    case 3: return launch<T, 3>(g, ax, a, s);
    case 4: return launch<T, 4>(g, ax, a, s);
    case 6: return launch<T, 6>(g, ax, a, s);
    case 8: return launch<T, 8>(g, ax, a, s);
    case 12: return launch<T, 12>(g, ax, a, s);
    case 16: return launch<T, 16>(g, ax, a, s);
    case 24: return launch<T, 24>(g, ax, a, s);
    case 32: return launch<T, 32>(g, ax, a, s);
    default: return cudaErrorInvalidValue;
  }
}

template cudaError_t wypass<double>(const Geometry&, const DstAxis<double>&, const YPassArgs<double>&, cudaStream_t);
template cudaError_t wypass<float>(const Geometry&, const DstAxis<float>&, const YPassArgs<float>&, cudaStream_t);

}  // namespace ib
