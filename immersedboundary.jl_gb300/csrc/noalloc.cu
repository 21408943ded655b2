// Allocation-free Laplacian inverse (ib_op_laplacian_inv_noalloc, include/ibgb300_ops.h).
//
// Some callers cannot call cudaMalloc in the loop that solves: programs whose device memory is
// owned by another allocator or memory pool (a Julia or Python host that hands this library
// only the arrays it already owns), and time-critical loops that must not pay for an
// allocation's implicit synchronisation of the whole device.  ib_op_laplacian_inv allocates its
// work buffer on every call; this variant keeps that work buffer in a fixed array compiled into
// the library instead.
//
// The array is a file-scope __device__ variable of kNoAllocMaxValues FP64 values (32 MiB).
// Every GPU that loads the library holds it until the process exits.  In host code its name
// only stands in for the symbol and is not a device address; the entry point looks up the
// device address once per device (cudaGetSymbolAddress, on the first call made on that
// device, with that device current) and passes that address to the kernels.  That first call
// on a device should come before any stream capture.
//
// All calls share the one array and it keeps the last call's contents.  The solve overwrites
// every value it reads before reading it, so nothing needs clearing; but calls that overlap on
// the GPU (other streams, other threads, other handles on the same device) race on it.
#include "ib_common.cuh"
#include "ibgb300_ops.h"

#include <mutex>

namespace {

constexpr size_t kNoAllocMaxValues = (size_t)1 << 22;  // 4,194,304 doubles = 32 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_work[kNoAllocMaxValues];

std::mutex g_mu;
double* g_work_addr[kMaxDevices] = {};

// Device address of g_noalloc_work on the current device (looked up on first use).
cudaError_t work_address(int device, double** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_work_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_work);
    if (e != cudaSuccess) return e;
    g_work_addr[device] = static_cast<double*>(p);
  }
  *out = g_work_addr[device];
  return cudaSuccess;
}

}  // namespace

extern "C" int ib_op_laplacian_inv_noalloc(ib_handle* h, int32_t batch, const double* b, double* x) {
  ib::LapView v;
  if (!ib_handle_lap_view(h, &v) || batch < 1 || !b || !x) return IB_ERR_INVALID;
  if ((size_t)batch * (size_t)v.g.nG > kNoAllocMaxValues)
    return ib_handle_fail(h, IB_ERR_INVALID,
                          "ib_op_laplacian_inv_noalloc: batch * (nx-1)*(ny-1) exceeds the 4194304-value work array");
  cudaError_t e = cudaSetDevice(v.device);
  double* w = nullptr;
  if (e == cudaSuccess) e = work_address(v.device, &w);
  if (e != cudaSuccess) return ib_handle_fail(h, IB_ERR_CUDA, cudaGetErrorString(e));
  // x = F2D(mlap .* F2D(b)): x pass into the fixed work array, y pass in place, x pass out
  ib::XArgs xa{};
  xa.in = b;
  xa.out = w;
  xa.batch = batch;
  xa.stride = v.g.nG;
  xa.pro = ib::kProLoad;
  xa.epi = ib::kEpiStore;
  e = ib::xpass<double, double, double>(v.g, v.ax, xa, v.stream);
  if (e == cudaSuccess) {
    ib::YPassArgs<double> ya{};
    ya.in1 = w;
    ya.out = w;
    ya.batch = batch;
    ya.stride = v.g.nG;
    ya.m1 = v.mlap;
    ya.mstride = 0;
    ya.op = ib::SpecOp::kScale;
    e = ib::ypass<double>(v.g, v.ay, ya, v.stream);
  }
  if (e == cudaSuccess) {
    ib::XArgs xb = xa;
    xb.in = w;
    xb.out = x;
    e = ib::xpass<double, double, double>(v.g, v.ax, xb, v.stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  if (e != cudaSuccess) return ib_handle_fail(h, IB_ERR_CUDA, cudaGetErrorString(e));
  return IB_OK;
}
