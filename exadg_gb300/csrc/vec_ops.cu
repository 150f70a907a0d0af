// Streaming vector kernels: precision conversion and fills.
#include "internal.h"

namespace exg {

template <class S, class D>
__global__ void convert_kernel(const S* __restrict__ s, D* __restrict__ d, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (; i < n; i += stride) d[i] = (D)s[i];
}

template <class T>
__global__ void fill_kernel(T* __restrict__ x, T v, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (; i < n; i += stride) x[i] = v;
}

static unsigned grid_for(long long n) {
  long long b = (n + 255) / 256;
  return (unsigned)(b < 152 * 32 ? (b < 1 ? 1 : b) : 152 * 32);
}

void vec_copy_convert(const void* src, int sp, void* dst, int dp, long long n, cudaStream_t s) {
  bool sd = sp != EXG_PREC_F32, dd = dp != EXG_PREC_F32;
  if (sd && dd)
    convert_kernel<double, double><<<grid_for(n), 256, 0, s>>>((const double*)src, (double*)dst, n);
  else if (sd && !dd)
    convert_kernel<double, float><<<grid_for(n), 256, 0, s>>>((const double*)src, (float*)dst, n);
  else if (!sd && dd)
    convert_kernel<float, double><<<grid_for(n), 256, 0, s>>>((const float*)src, (double*)dst, n);
  else
    convert_kernel<float, float><<<grid_for(n), 256, 0, s>>>((const float*)src, (float*)dst, n);
  EXG_CUDA(cudaGetLastError());
}

void vec_fill(void* x, int prec, double v, long long n, cudaStream_t s) {
  if (prec == EXG_PREC_F32)
    fill_kernel<float><<<grid_for(n), 256, 0, s>>>((float*)x, (float)v, n);
  else
    fill_kernel<double><<<grid_for(n), 256, 0, s>>>((double*)x, v, n);
  EXG_CUDA(cudaGetLastError());
}

}  // namespace exg
