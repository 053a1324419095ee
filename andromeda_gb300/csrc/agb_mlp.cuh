// MLP surrogate (nin -> nh -> nh -> nh -> nout, SiLU) on BF16 tensor cores.
#pragma once
#include "agb_common.cuh"
#include <string>

namespace agb {

struct Mlp {
  int device = 0;
  cudaStream_t s = nullptr;
  int nin = 5, nh = 256, nout = 21;
  float* params = nullptr;  // W1 [nh][nin], b1, W2 [nh][nh], b2, W3, b3, W4 [nout][nh], b4 (FP32 master copy)
  float* grads = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  float* norm = nullptr;    // x_mean[nin], x_std[nin], y_mean[nout], y_std[nout]
  float* ws = nullptr;      // activations of ws_rows rows
  double* part = nullptr;   // loss partial sums
  void* wt = nullptr;       // BF16 hi/lo weights packed for the tcgen05 inference kernel (nh = 256, nin <= 16,
                            // nout <= 32)
  int* tc_err = nullptr;    // bounded-wait flag of the tcgen05 inference kernel
  int ws_rows = 0;
  int step = 0;
  long launches = 0;
  std::string err;

  ~Mlp();
  void release();
  int64_t nparams() const;
  void offsets(int64_t o[8]) const;
  bool init(int dev, uint64_t seed, cudaStream_t st);
  bool ensure_ws(int rows);
  void load_inputs(int rows, const float* X_dev);   // normalised into the workspace
  void forward(int rows, bool train, bool split);
  void backward(int rows, const float* T_dev, bool split);  // gradients into grads, loss partials into part
  void adam(float lr);
  void output(int rows, float* Y_dev);              // de-normalised outputs of the last forward
  bool infer(int rows, const float* X_dev, float* Y_dev);  // fused split-BF16 inference on tcgen05 (one kernel)
  double loss_sum(int rows);                        // sum of squared normalised errors of the last backward
};

}  // namespace agb
