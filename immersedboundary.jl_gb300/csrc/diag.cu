// FP64 / FP32 pipe throughput probe (ib_measure_fp_peaks, include/ibgb300_diag.h).
#include "ib_common.cuh"
#include "ibgb300_diag.h"

#include <cuda_profiler_api.h>

namespace {

template <typename T>
__global__ void k_fma_chains(T* out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = (T)(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = x[k] * a + b;
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
double probe(int sms, int iters, cudaStream_t st) {
  const int blocks = sms * 8, threads = 256;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return -1.0;
  k_fma_chains<T><<<blocks, threads, 0, st>>>(out, 16, (T)0.999, (T)0.001);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, st);
  k_fma_chains<T><<<blocks, threads, 0, st>>>(out, iters, (T)0.999, (T)0.001);
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double flops = 2.0 * 8 * (double)iters * blocks * threads;
  return ms > 0 ? flops / (ms * 1e-3) / 1e12 : -1.0;
}

}  // namespace

extern "C" int ib_measure_fp_peaks(int32_t device, double* fp64_tflops, double* fp32_tflops) {
  ib::DeviceGuard dev_guard_(device);
  if (dev_guard_.err != cudaSuccess) return IB_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaStream_t st;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return IB_ERR_CUDA;
  const double d = probe<double>(sms, 20000, st);
  const double f = probe<float>(sms, 200000, st);
  cudaStreamDestroy(st);
  if (fp64_tflops) *fp64_tflops = d;
  if (fp32_tflops) *fp32_tflops = f;
  return (d > 0 && f > 0 && cudaGetLastError() == cudaSuccess) ? IB_OK : IB_ERR_CUDA;
}

extern "C" int ib_profiler_start(void) { return cudaProfilerStart() == cudaSuccess ? IB_OK : IB_ERR_CUDA; }
extern "C" int ib_profiler_stop(void) { return cudaProfilerStop() == cudaSuccess ? IB_OK : IB_ERR_CUDA; }
