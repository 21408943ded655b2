// Allocation-free Laplacian inverse (ib_op_laplacian_inv_noalloc, include/ibgb300_ops.h).
//
// Some callers cannot call cudaMalloc in the loop that solves: programs whose device memory is
// owned by another allocator or memory pool (a Julia or Python host that hands this library
// only the arrays it already owns), and time-critical loops that must not pay for an
// allocation's implicit synchronisation of the whole device.  ib_op_laplacian_inv allocates its
// work buffer on every call; this variant keeps that work buffer in a fixed array compiled into
// the library instead, and runs the same transform kernels as ib_op_laplacian_inv on the same
// handle (warp-per-line passes where the handle uses them, Stockham passes otherwise).
//
// The array is a file-scope __device__ variable of kNoAllocMaxValues FP64 values (32 MiB).
// Every GPU that loads the library holds it until the process exits.  In host code its name
// only stands in for the symbol and is not a device address; every call looks up the device
// address (cudaGetSymbolAddress, with the handle's device current; the lookup does not
// synchronise) and passes that address to the kernels, so a re-created context cannot leave a
// stale address behind.  The first call on a device also loads the module there, so it should
// come before any stream capture.
//
// All calls share the one array and it keeps the last call's contents.  The solve overwrites
// every value it reads before reading it, so nothing needs clearing; but calls that overlap on
// the GPU (other streams, other threads, other handles on the same device) race on it.
#include "ib_common.cuh"
#include "ibgb300_ops.h"

#include <mutex>

namespace {

constexpr size_t kNoAllocMaxValues = (size_t)1 << 22;  // 4,194,304 doubles = 32 MiB

static __device__ __align__(256) double g_noalloc_work[kNoAllocMaxValues];

}  // namespace

extern "C" int ib_op_laplacian_inv_noalloc(ib_handle* h, int32_t batch, const double* b, double* x) {
  ib::LapView v;
  if (!ib_handle_lap_view(h, &v) || batch < 1 || !b || !x) return IB_ERR_INVALID;
  if ((size_t)batch * (size_t)v.g.nG > kNoAllocMaxValues)
    return ib_handle_fail(h, IB_ERR_INVALID,
                          "ib_op_laplacian_inv_noalloc: batch * (nx-1)*(ny-1) exceeds the 4194304-value work array");
  ib::DeviceGuard guard(v.device);
  cudaError_t e = guard.err;
  void* wp = nullptr;
  if (e == cudaSuccess) e = cudaGetSymbolAddress(&wp, g_noalloc_work);
  if (e != cudaSuccess) return ib_handle_fail(h, IB_ERR_CUDA, cudaGetErrorString(e));
  double* w = static_cast<double*>(wp);
  // x = F2D(mlap .* F2D(b)): x pass into the fixed work array, y pass in place, x pass out
  ib::XArgs xa{};
  xa.in = b;
  xa.out = w;
  xa.batch = batch;
  xa.stride = v.g.nG;
  xa.bcfac = 1.0;
  xa.pro = ib::kProLoad;
  xa.epi = ib::kEpiStore;
  ib::YPassArgs<double> ya{};
  ya.in1 = w;
  ya.out = w;
  ya.batch = batch;
  ya.stride = v.g.nG;
  ya.m1 = v.mlap;
  ya.mstride = 0;
  ya.op = ib::SpecOp::kScale;
  ib::XArgs xb = xa;
  xb.in = w;
  xb.out = x;
  if (v.wdst) {
    // warp-per-line passes; the work array holds the transposed intermediate
    e = ib::wx_fwd<double, double>(v.g, v.ax, xa, v.stream);
    if (e == cudaSuccess) e = ib::wypass<double>(v.g, v.ay, ya, v.stream);
    if (e == cudaSuccess) e = ib::wx_inv<double, double>(v.g, v.ax, xb, v.stream);
  } else {
    e = ib::xpass<double, double, double>(v.g, v.ax, xa, v.stream);
    if (e == cudaSuccess) e = ib::ypass<double>(v.g, v.ay, ya, v.stream);
    if (e == cudaSuccess) e = ib::xpass<double, double, double>(v.g, v.ax, xb, v.stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  if (e != cudaSuccess) return ib_handle_fail(h, IB_ERR_CUDA, cudaGetErrorString(e));
  return IB_OK;
}
