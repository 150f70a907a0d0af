// Solver-side kernels: CG vector updates with fused FP64 reductions, Chebyshev recurrences,
// DG p/h transfers, and the single-CTA coarse-grid CG.
//
// Reductions are deterministic: every block writes one partial sum, the last block to finish
// adds the partials in index order (no floating-point atomics).
#include <cuda_runtime.h>

#include "internal.h"
#include "solver_kernels.h"

namespace exg {

static constexpr int RED_BLOCKS = 608;  // 4 x 152 SMs
static constexpr int RED_THREADS = 256;

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;  // valid in thread 0
}

// last-block finalisation of a partial-sum reduction into out[slot]
__device__ __forceinline__ void finish_reduction(double partial, Reduction red, int slot) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    red.partials[slot * RED_BLOCKS + blockIdx.x] = partial;
    __threadfence();
    unsigned int t = atomicAdd(&red.counter[slot], 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __shared__ double sh[32];
    double v = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) v += ((volatile double*)red.partials)[slot * RED_BLOCKS + i];
    v = block_sum(v, sh);
    if (threadIdx.x == 0) {
      red.out[slot] = v;
      red.counter[slot] = 0;
    }
  }
}

Reduction Reduction::create() {
  Reduction r;
  EXG_CUDA(cudaMalloc(&r.partials, sizeof(double) * RED_BLOCKS * kSlots));
  EXG_CUDA(cudaMalloc(&r.out, sizeof(double) * kSlots));
  EXG_CUDA(cudaMalloc(&r.counter, sizeof(unsigned int) * kSlots));
  EXG_CUDA(cudaMemset(r.counter, 0, sizeof(unsigned int) * kSlots));
  EXG_CUDA(cudaMemset(r.out, 0, sizeof(double) * kSlots));
  return r;
}
void Reduction::destroy() {
  if (partials) cudaFree(partials);
  if (out) cudaFree(out);
  if (counter) cudaFree(counter);
  partials = out = nullptr;
  counter = nullptr;
}

// ------------------------------------------------------------------------------------------------
template <class T>
__global__ void dot_kernel(const T* __restrict__ x, const T* __restrict__ y, long long n, Reduction red, int slot) {
  __shared__ double sh[32];
  double s = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    s += (double)x[i] * (double)y[i];
  s = block_sum(s, sh);
  finish_reduction(s, red, slot);
}

// r = b - v (or r = b), slot <- |r|^2
template <class T>
__global__ void residual_kernel(const T* __restrict__ b, const T* __restrict__ v, T* __restrict__ r, long long n,
                                Reduction red, int slot) {
  __shared__ double sh[32];
  double s = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    T ri = v ? b[i] - v[i] : b[i];
    r[i] = ri;
    s += (double)ri * (double)ri;
  }
  s = block_sum(s, sh);
  finish_reduction(s, red, slot);
}

// z = d .* r (Jacobi) or z = r; slot <- r.z
template <class T>
__global__ void precond_dot_kernel(const T* __restrict__ d, const T* __restrict__ r, T* __restrict__ z, long long n,
                                   Reduction red, int slot) {
  __shared__ double sh[32];
  double s = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    T zi = d ? d[i] * r[i] : r[i];
    z[i] = zi;
    s += (double)r[i] * (double)zi;
  }
  s = block_sum(s, sh);
  finish_reduction(s, red, slot);
}

// p = z + beta p (beta = 0 on the first iteration)
template <class T>
__global__ void p_update_kernel(const T* __restrict__ z, T* __restrict__ p, T beta, bool first, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = first ? z[i] : z[i] + beta * p[i];
}

// x += alpha p; r -= alpha v; slot <- |r|^2
template <class T>
__global__ void xr_update_kernel(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                                 const T* __restrict__ v, T alpha, long long n, Reduction red, int slot) {
  __shared__ double sh[32];
  double s = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    T ri = r[i] - alpha * v[i];
    r[i] = ri;
    s += (double)ri * (double)ri;
  }
  s = block_sum(s, sh);
  finish_reduction(s, red, slot);
}

template <class T>
void dot(const T* x, const T* y, long long n, Reduction& red, int slot, cudaStream_t s) {
  dot_kernel<T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(x, y, n, red, slot);
  EXG_CUDA(cudaGetLastError());
}
template <class T>
void residual(const T* b, const T* v, T* r, long long n, Reduction& red, int slot, cudaStream_t s) {
  residual_kernel<T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(b, v, r, n, red, slot);
  EXG_CUDA(cudaGetLastError());
}
template <class T>
void precond_dot(const T* d, const T* r, T* z, long long n, Reduction& red, int slot, cudaStream_t s) {
  precond_dot_kernel<T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(d, r, z, n, red, slot);
  EXG_CUDA(cudaGetLastError());
}
template <class T>
void p_update(const T* z, T* p, double beta, bool first, long long n, cudaStream_t s) {
  p_update_kernel<T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(z, p, (T)beta, first, n);
  EXG_CUDA(cudaGetLastError());
}
template <class T>
void xr_update(T* x, T* r, const T* p, const T* v, double alpha, long long n, Reduction& red, int slot,
               cudaStream_t s) {
  xr_update_kernel<T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(x, r, p, v, (T)alpha, n, red, slot);
  EXG_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------------------------------------
// Chebyshev recurrences (deal.II PreconditionChebyshev, first kind; chebyshev_smoother.h:79-210)
//   mode 0: x = f2 d.*b                                  (vmult, iteration 0, zero start)
//   mode 1: old = x; x = x + f2 d.*(b - t)               (step, first update)
//   mode 2: old = x; x = (1+f1) x + f2 d.*(b - t)        (second update after a zero start)
//   mode 3: new = (1+f1) x - f1 old + f2 d.*(b - t); old = x; x = new
// ------------------------------------------------------------------------------------------------
template <class T>
__global__ void cheb_kernel(int mode, T* __restrict__ x, T* __restrict__ old, const T* __restrict__ b,
                            const T* __restrict__ t, const T* __restrict__ d, T f1, T f2, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (mode == 0) {
      x[i] = f2 * (d[i] * b[i]);
      continue;
    }
    T xi = x[i];
    T pr = d[i] * (b[i] - t[i]);
    T xn;
    if (mode == 1)
      xn = xi + f2 * pr;
    else if (mode == 2)
      xn = (T(1) + f1) * xi + f2 * pr;
    else
      xn = (T(1) + f1) * xi - f1 * old[i] + f2 * pr;
    old[i] = xi;
    x[i] = xn;
  }
}

template <class T>
void chebyshev_update(int mode, T* x, T* old, const T* b, const T* t, const T* d, double f1, double f2, long long n,
                      cudaStream_t s) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  cheb_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(mode, x, old, b, t, d, (T)f1, (T)f2, n);
  EXG_CUDA(cudaGetLastError());
}

// t = b - t
template <class T>
__global__ void rsub_kernel(const T* __restrict__ b, T* __restrict__ t, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    t[i] = b[i] - t[i];
}
template <class T>
void rsub(const T* b, T* t, long long n, cudaStream_t s) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  rsub_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(b, t, n);
  EXG_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------------------------------------
// DG transfers (MGTwoLevelTransfer, element-local interpolation; restriction = transpose)
// ------------------------------------------------------------------------------------------------
template <class T>
__global__ void prolongate_kernel(TransferParams P, const T* __restrict__ coarse, T* __restrict__ fine, long long n_fine) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_fine) return;
  const int nf = P.nf, nc = P.nc, nf3 = nf * nf * nf, nc3 = nc * nc * nc;
  long long cf = g / nf3;
  int loc = (int)(g - cf * nf3);
  int ix[3] = {loc % nf, (loc / nf) % nf, loc / (nf * nf)};
  int ci[3] = {(int)(cf % P.Nf[0]), (int)((cf / P.Nf[0]) % P.Nf[1]), (int)(cf / ((long long)P.Nf[0] * P.Nf[1]))};
  int ch[3] = {0, 0, 0};
  long long cc = cf;
  if (P.is_h) {
    for (int e = 0; e < 3; ++e) ch[e] = ci[e] & 1;
    cc = (ci[0] >> 1) + (long long)P.Nc[0] * ((ci[1] >> 1) + (long long)P.Nc[1] * (ci[2] >> 1));
  }
  const T* u = coarse + cc * nc3;
  const double* P0 = P.P[ch[0]] + ix[0] * nc;
  const double* P1 = P.P[ch[1]] + ix[1] * nc;
  const double* P2 = P.P[ch[2]] + ix[2] * nc;
  double s = 0;
  for (int c2 = 0; c2 < nc; ++c2)
    for (int c1 = 0; c1 < nc; ++c1) {
      double w = P2[c2] * P1[c1];
      const T* ul = u + (c2 * nc + c1) * nc;
      for (int c0 = 0; c0 < nc; ++c0) s += w * P0[c0] * (double)ul[c0];
    }
  fine[g] += (T)s;
}

template <class T>
__global__ void restrict_kernel(TransferParams P, const T* __restrict__ fine, T* __restrict__ coarse, long long n_coarse) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_coarse) return;
  const int nf = P.nf, nc = P.nc, nf3 = nf * nf * nf, nc3 = nc * nc * nc;
  long long cc = g / nc3;
  int loc = (int)(g - cc * nc3);
  int jx[3] = {loc % nc, (loc / nc) % nc, loc / (nc * nc)};
  int ci[3] = {(int)(cc % P.Nc[0]), (int)((cc / P.Nc[0]) % P.Nc[1]), (int)(cc / ((long long)P.Nc[0] * P.Nc[1]))};
  double s = 0;
  int nch = P.is_h ? 8 : 1;
  for (int c8 = 0; c8 < nch; ++c8) {
    int ch[3] = {c8 & 1, (c8 >> 1) & 1, (c8 >> 2) & 1};
    long long cf = cc;
    if (P.is_h)
      cf = (2 * ci[0] + ch[0]) + (long long)P.Nf[0] * ((2 * ci[1] + ch[1]) + (long long)P.Nf[1] * (2 * ci[2] + ch[2]));
    else
      ch[0] = ch[1] = ch[2] = 0;
    const T* u = fine + cf * nf3;
    for (int i2 = 0; i2 < nf; ++i2)
      for (int i1 = 0; i1 < nf; ++i1) {
        double w = P.P[ch[2]][i2 * nc + jx[2]] * P.P[ch[1]][i1 * nc + jx[1]];
        const T* ul = u + (i2 * nf + i1) * nf;
        for (int i0 = 0; i0 < nf; ++i0) s += w * P.P[ch[0]][i0 * nc + jx[0]] * (double)ul[i0];
      }
  }
  coarse[g] += (T)s;
}

template <class T>
void prolongate_add(const TransferParams& P, const T* coarse, T* fine, cudaStream_t s) {
  long long n = (long long)P.Nf[0] * P.Nf[1] * P.Nf[2] * P.nf * P.nf * P.nf;
  prolongate_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, coarse, fine, n);
  EXG_CUDA(cudaGetLastError());
}
template <class T>
void restrict_add(const TransferParams& P, const T* fine, T* coarse, cudaStream_t s) {
  long long n = (long long)P.Nc[0] * P.Nc[1] * P.Nc[2] * P.nc * P.nc * P.nc;
  restrict_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, fine, coarse, n);
  EXG_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------------------------------------
// coarse CG + point Jacobi in one CTA (MGCoarseKrylov, coarse_grid_solvers.h:157-224).  The dense
// coarse matrix is assembled at setup.  Iterations are bounded by max_iter.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ double cta_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
  return r;  // valid in all threads
}

template <class T, class CT>
__global__ void coarse_cg_kernel(const CT* __restrict__ A, const CT* __restrict__ invd, const T* __restrict__ rhs,
                                 T* __restrict__ xout, CT* __restrict__ xstate, int n, double rel_tol, double abs_tol,
                                 int max_iter, int singular, long long* __restrict__ its_counter) {
  extern __shared__ __align__(16) unsigned char sm[];
  CT* x = reinterpret_cast<CT*>(sm);
  CT* r = x + n;
  CT* z = r + n;
  CT* p = z + n;
  CT* v = p + n;
  __shared__ double sh[32];
  const int tid = threadIdx.x, nt = blockDim.x;
  // r = src (mean removed if singular)
  double mean = 0;
  if (singular) {
    double s = 0;
    for (int i = tid; i < n; i += nt) s += (double)rhs[i];
    mean = cta_sum(s, sh) / n;
  }
  for (int i = tid; i < n; i += nt) {
    x[i] = xstate[i];
    z[i] = (CT)((double)rhs[i] - mean);  // b
  }
  __syncthreads();
  // r = b - A x
  bool xzero = true;
  for (int i = 0; i < n; ++i)
    if (x[i] != CT(0)) {
      xzero = false;
      break;
    }
  double rr = 0;
  for (int i = tid; i < n; i += nt) {
    CT s = 0;
    if (!xzero)
      for (int j = 0; j < n; ++j) s += A[(long long)j * n + i] * x[j];  // A symmetric: coalesced columns
    r[i] = z[i] - s;
    rr += (double)r[i] * (double)r[i];
  }
  double rn = sqrt(cta_sum(rr, sh));
  const double tol = fmax(abs_tol, rel_tol * rn);
  int it = 0;
  double rho_old = 1;
  while (rn > tol && it < max_iter) {
    ++it;
    double rz = 0;
    for (int i = tid; i < n; i += nt) {
      z[i] = invd[i] * r[i];
      rz += (double)r[i] * (double)z[i];
    }
    double rho = cta_sum(rz, sh);
    double beta = it == 1 ? 0.0 : rho / rho_old;
    for (int i = tid; i < n; i += nt) p[i] = it == 1 ? z[i] : z[i] + (CT)beta * p[i];
    __syncthreads();
    double pv = 0;
    for (int i = tid; i < n; i += nt) {
      CT s = 0;
      for (int j = 0; j < n; ++j) s += A[(long long)j * n + i] * p[j];
      v[i] = s;
      pv += (double)p[i] * (double)s;
    }
    pv = cta_sum(pv, sh);
    double alpha = rho / pv;
    double rr2 = 0;
    for (int i = tid; i < n; i += nt) {
      x[i] += (CT)alpha * p[i];
      r[i] -= (CT)alpha * v[i];
      rr2 += (double)r[i] * (double)r[i];
    }
    rn = sqrt(cta_sum(rr2, sh));
    rho_old = rho;
  }
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    xstate[i] = x[i];
    xout[i] = (T)x[i];
  }
  if (tid == 0) its_counter[0] += it;
}

template <class T, class CT>
void coarse_cg(const CT* A, const CT* invd, const T* rhs, T* x, CT* xstate, int n, double rel_tol, double abs_tol,
               int max_iter, int singular, long long* its, cudaStream_t s) {
  size_t smem = 5 * (size_t)n * sizeof(CT);
  auto k = coarse_cg_kernel<T, CT>;
  static int attr_bytes = 0;
  if ((int)smem > attr_bytes) {
    EXG_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_bytes = (int)smem;
  }
  k<<<1, 1024, smem, s>>>(A, invd, rhs, x, xstate, n, rel_tol, abs_tol, max_iter, singular, its);
  EXG_CUDA(cudaGetLastError());
}

// identity columns for the coarse-matrix assembly: e[j][i] = (i == j)
template <class T>
__global__ void identity_kernel(T* e, int n) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < (long long)n * n) e[g] = (g / n == g % n) ? T(1) : T(0);
}
template <class T>
void identity(T* e, int n, cudaStream_t s) {
  long long t = (long long)n * n;
  identity_kernel<T><<<(unsigned)((t + 255) / 256), 256, 0, s>>>(e, n);
  EXG_CUDA(cudaGetLastError());
}

// explicit instantiations
#define INST(T)                                                                                          \
  template void dot<T>(const T*, const T*, long long, Reduction&, int, cudaStream_t);                    \
  template void residual<T>(const T*, const T*, T*, long long, Reduction&, int, cudaStream_t);           \
  template void precond_dot<T>(const T*, const T*, T*, long long, Reduction&, int, cudaStream_t);        \
  template void p_update<T>(const T*, T*, double, bool, long long, cudaStream_t);                         \
  template void xr_update<T>(T*, T*, const T*, const T*, double, long long, Reduction&, int, cudaStream_t); \
  template void chebyshev_update<T>(int, T*, T*, const T*, const T*, const T*, double, double, long long, cudaStream_t); \
  template void rsub<T>(const T*, T*, long long, cudaStream_t);                                           \
  template void prolongate_add<T>(const TransferParams&, const T*, T*, cudaStream_t);                     \
  template void restrict_add<T>(const TransferParams&, const T*, T*, cudaStream_t);                       \
  template void identity<T>(T*, int, cudaStream_t);
INST(float)
INST(double)
template void coarse_cg<float, float>(const float*, const float*, const float*, float*, float*, int, double, double,
                                      int, int, long long*, cudaStream_t);
template void coarse_cg<float, double>(const double*, const double*, const float*, float*, double*, int, double,
                                       double, int, int, long long*, cudaStream_t);
template void coarse_cg<double, double>(const double*, const double*, const double*, double*, double*, int, double,
                                        double, int, int, long long*, cudaStream_t);

}  // namespace exg
