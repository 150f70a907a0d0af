// Cell-patch CNN of the learned initial guess (cnn.cu).
#pragma once

#include <cuda_runtime.h>

#include "internal.h"

struct exg_cnn {
  int N[3];
  long long n_cells;
  int c_in, c_hid, c_out;
  long long off[7];  // W1, b1, W2, b2, W3, b3, W4 (linear skip) offsets into params
  long long n_params;
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
  float *a1 = nullptr, *p1 = nullptr, *a2 = nullptr, *p2 = nullptr, *y = nullptr;
  float *g2 = nullptr, *g1 = nullptr, *gy = nullptr, *wt = nullptr;
  float *wpart = nullptr, *bpart = nullptr, *loss_part = nullptr, *bskip = nullptr;
  int chunk = 256, n_chunks = 0;
  long long step = 0;

  exg_cnn(const int n[3], int cin, int chid, int cout, unsigned long long seed);
  ~exg_cnn();
  void forward(const float* x, float* out, bool keep, cudaStream_t s);
  void backward(const float* x, const float* gout, cudaStream_t s);
  float loss_and_grad(const float* x, const float* target, cudaStream_t s);
  void adam(float lr, float grad_scale, cudaStream_t s);

 private:
  void wgrad(int K, const float* in, const float* g, int cin, int cout, float* gW, float* gb, cudaStream_t s);
};
