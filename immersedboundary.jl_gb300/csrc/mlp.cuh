// Learned warm start of the moving-body Schur CG (mlp.cu): network, sample store, training.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace ib {
namespace learn {

constexpr int kMaxBatch = 512;  // rows per training minibatch

struct Mlp {
  // layer widths dims[0] (features) .. dims[nl] (forces); W_l is [dims[l+1]][dims[l]] row-major
  std::vector<int> dims;
  int nl = 0;
  std::vector<int64_t> woff, boff;  // offsets of W_l and b_l in the parameter vector
  int64_t nparam = 0, nweights = 0;
  float* master = nullptr;          // FP32 parameters (Adam updates these)
  float* grad = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  __nv_bfloat16* wbf = nullptr;     // BF16 copy used by the products (biases unused there)
  std::vector<float*> act, dact;    // per layer activations / their gradients, kMaxBatch rows
  float* ybatch = nullptr;
  // samples: raw features and F_n, a ring of `cap` rows
  float *xs = nullptr, *ys = nullptr;
  int cap = 0, count = 0, next = 0;
  float *feat = nullptr, *featn = nullptr;  // raw features of the current step
  float *mu_x = nullptr, *sd_x = nullptr, *mu_y = nullptr, *sd_y = nullptr;
  double* loss = nullptr;
  int* idx = nullptr;
  int* d_next = nullptr;  // device copy of next (the recording kernel advances it)
  bool trained = false;
  double blend = 1.0;    // weight of the network's correction (validated at training)
  double val_rel = -1;   // held-out squared error relative to plain extrapolation's (-1: none)
  std::vector<int> val_rows;  // sample slots of the held-out rows of the last training, oldest first
  int adam_t = 0;
  cudaStream_t stream = nullptr;
  int* status = nullptr;  // device flag set when a tensor-core product gave up waiting
  std::vector<void*> allocs;

  ~Mlp() { release(); }
  cudaError_t init(int din, int dout, int hidden, int nhidden, int capacity, uint64_t seed, cudaStream_t s,
                   int* status_flag);
  void release();
  cudaError_t sync_bf16();
  cudaError_t forward(int b);
  cudaError_t backward(int b);
  cudaError_t adam_step(float lr);
  // per step: raw features from device kinematics and force history; record F_n; prediction
  cudaError_t features(const double* kin, int nkin, const double* f1, const double* f2, int nf);
  cudaError_t record(const double* fn);         // record_enqueue + record_commit
  cudaError_t record_enqueue(const double* fn); // the device side (slot index on the device)
  void record_commit();                         // the host mirror of count / next
  cudaError_t predict(const double* f1, const double* f2, double* fb);
  cudaError_t train(int epochs, int batch, float lr, uint64_t seed, double* final_loss);
  // the network's corrections q and the targets t (F_n minus its extrapolation) of the most
  // recent held-out rows, denormalised, row-major [rows][nf] in FP64; at most max_rows rows
  cudaError_t heldout(double* q, double* t, int max_rows, int* rows);
  // loss and parameter gradients of the raw network on host rows (normalised inputs/targets)
  cudaError_t gradients(int b, const float* x_host, const float* y_host, float* grad_host, double* loss_host);
};

}  // namespace learn
}  // namespace ib
