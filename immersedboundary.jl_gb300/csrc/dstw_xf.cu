// Line-parallel forward x pass: prologue, S_x, transposed store (kernels in dstw_x.cuh).
#include "dstw_x.cuh"

namespace ib {

template <typename T, typename Tin>
cudaError_t wx_fwd(const Geometry& g, const DstAxis<T>& ax, const XArgs& a, cudaStream_t s) {
  if (ax.n != g.nx || !ax.wP) return cudaErrorInvalidValue;
  if (a.batch <= 0) return cudaSuccess;
  ProfScope prof(kClassXPass, s);
  switch (ax.wNL * 100 + ax.wP) {
#define IB_WCASE(NL, P) \
  case NL * 100 + P: return fwd_p<T, Tin, P, NL>(g, ax, a, s);
    IB_WDST_COMBOS(IB_WCASE)
#undef IB_WCASE
    default: return cudaErrorInvalidValue;
  }
}

// FP64 path: double in.  Mixed path: float-float input, FP32 transforms.
template cudaError_t wx_fwd<double, double>(const Geometry&, const DstAxis<double>&, const XArgs&, cudaStream_t);
template cudaError_t wx_fwd<float, df64>(const Geometry&, const DstAxis<float>&, const XArgs&, cudaStream_t);

}  // namespace ib
