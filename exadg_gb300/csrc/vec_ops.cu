// Streaming vector kernels: precision conversion and fills; per-device kernel attributes.
#include <map>
#include <mutex>
#include <utility>

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

// FMA throughput probe: independent chains of a*x+b per thread, bounded iteration count
template <class T, int CHAINS>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
  T acc[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) acc[c] = (T)(threadIdx.x + c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) acc[c] = acc[c] * a + b;
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) s += acc[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class T>
static double fma_rate(int sms, cudaStream_t s) {
  const int blocks = sms * 8, threads = 256, iters = sizeof(T) == 8 ? 512 : 4096;
  T* out = nullptr;
  EXG_CUDA(cudaMalloc(&out, sizeof(T) * blocks * threads));
  cudaEvent_t e0, e1;
  EXG_CUDA(cudaEventCreate(&e0));
  EXG_CUDA(cudaEventCreate(&e1));
  fma_probe_kernel<T, 8><<<blocks, threads, 0, s>>>(out, 64, (T)0.999, (T)1e-3);
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    EXG_CUDA(cudaEventRecord(e0, s));
    fma_probe_kernel<T, 8><<<blocks, threads, 0, s>>>(out, iters, (T)0.999, (T)1e-3);
    EXG_CUDA(cudaEventRecord(e1, s));
    EXG_CUDA(cudaEventSynchronize(e1));
    float ms;
    EXG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    best = ms < best ? ms : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return 2.0 * 8 * (double)iters * blocks * threads / (best * 1e-3) / 1e12;  // TFLOP/s, FMA = 2
}

void ensure_smem_attr(const void* kernel, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> done;  // (kernel, device) -> bytes set
  int dev = 0;
  EXG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  int& have = done[{kernel, dev}];
  if (bytes > have) {
    EXG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    have = bytes;
  }
}

void device_fma_peaks(double* f64_tflops, double* f32_tflops, cudaStream_t s) {
  int dev = 0, sms = 0;
  EXG_CUDA(cudaGetDevice(&dev));
  EXG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (f64_tflops) *f64_tflops = fma_rate<double>(sms, s);
  if (f32_tflops) *f32_tflops = fma_rate<float>(sms, s);
}

}  // namespace exg
