// Warp-per-line y pass at the default occupancy (IB_WDST_YMINB resident blocks per SM) and the
// dispatcher between it and the 8-block variant of dstw_y8.cu (kernels in dstw_y.cuh).
#include "dstw_y.cuh"

#include <type_traits>

namespace ib {

extern template cudaError_t wypass_minb<float, 8>(const Geometry&, const DstAxis<float>&, const YPassArgs<float>&,
                                                 cudaStream_t);

template <typename T>
cudaError_t wypass(const Geometry& g, const DstAxis<T>& ax, const YPassArgs<T>& a, cudaStream_t s) {
  if (ax.n != g.ny || !ax.wP) return cudaErrorInvalidValue;
  if (a.batch <= 0) return cudaSuccess;
  ProfScope prof(kClassYPass, s);
  if constexpr (std::is_same<T, float>::value) {
    if (ax.wMinB == 8 && IB_WDST_YMINB != 8) return wypass_minb<float, 8>(g, ax, a, s);
  }
  return wypass_minb<T, IB_WDST_YMINB>(g, ax, a, s);
}

template cudaError_t wypass_minb<double, IB_WDST_YMINB>(const Geometry&, const DstAxis<double>&,
                                                       const YPassArgs<double>&, cudaStream_t);
template cudaError_t wypass_minb<float, IB_WDST_YMINB>(const Geometry&, const DstAxis<float>&, const YPassArgs<float>&,
                                                      cudaStream_t);
template cudaError_t wypass<double>(const Geometry&, const DstAxis<double>&, const YPassArgs<double>&, cudaStream_t);
template cudaError_t wypass<float>(const Geometry&, const DstAxis<float>&, const YPassArgs<float>&, cudaStream_t);

}  // namespace ib
