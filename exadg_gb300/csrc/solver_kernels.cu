// Solver-side kernels: CG vector updates with fused FP64 reductions, Chebyshev recurrences,
// DG p/h transfers, and the single-CTA coarse-grid CG.
//
// Reductions are deterministic: every block writes one partial sum, the last block to finish
// adds the partials in index order (no floating-point atomics).
#include <cuda_runtime.h>

#include <algorithm>

#include "epilogue.cuh"
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

// as xr_update_kernel with alpha read from device memory (graph-driven CG)
__global__ void xr_update_dev_kernel(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                                     const double* __restrict__ v, const double* __restrict__ alpha_ptr, long long n,
                                     Reduction red, int slot) {
  __shared__ double sh[32];
  const double alpha = *alpha_ptr;
  double s = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    double ri = r[i] - alpha * v[i];
    r[i] = ri;
    s += ri * ri;
  }
  s = block_sum(s, sh);
  finish_reduction(s, red, slot);
}

void xr_update_dev(double* x, double* r, const double* p, const double* v, const double* alpha, long long n,
                   Reduction& red, int slot, cudaStream_t s) {
  xr_update_dev_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(x, r, p, v, alpha, n, red, slot);
  EXG_CUDA(cudaGetLastError());
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
    T xn = cheb_point<T>(mode, xi, mode == 3 ? old[i] : T(0), b[i], t[i], d[i], f1, f2);
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
// DG transfers (MGTwoLevelTransfer, element-local interpolation; restriction = transpose), sum
// factorised: per fine cell the 3D interpolation P2 x P1 x P0 is applied as three 1D sweeps through
// shared memory (nf nc^3 + nf^2 nc^2 + nf^3 nc multiply-adds instead of nf^3 nc^3), in the
// multigrid's own number type.  A block handles G consecutive cells; for h-transfers the 1D matrix
// of each direction is the one of the cell's child position in its parent.
// ------------------------------------------------------------------------------------------------
// cells per block.  Large levels: enough fine values per block (~4096) to amortise the three
// barrier-separated sweeps, within 40 KB of static shared memory for the larger (restriction)
// footprint.  Small levels (fewer than 8 blocks per SM at that size): ~512 fine values per block.
template <int NF, int NC, class T>
struct TransferShape {
  static constexpr int per_cell = NF * NF * NF + NF * NF * NC + NF * NC * NC + NC * NC * NC;
  static constexpr int by_work = 4096 / (NF * NF * NF);
  static constexpr int by_smem = (40 * 1024 / (int)sizeof(T) - 2 * NF * NC) / per_cell;
  static constexpr int G0 = by_work < by_smem ? by_work : by_smem;
  static constexpr int large = G0 < 1 ? 1 : G0;
  static constexpr int small = 512 / (NF * NF * NF) < 1 ? 1 : 512 / (NF * NF * NF);
  static bool use_large(long long cells) { return cells >= (long long)large * 152 * 8; }
};

template <int NF, int NC, int G, class T>
__global__ void __launch_bounds__(256) prolongate_kernel(const __grid_constant__ TransferParams P,
                                                         const T* __restrict__ coarse, T* __restrict__ fine,
                                                         long long n_cells) {
  constexpr int nf = NF, nc = NC, nf2 = nf * nf, nf3 = nf2 * nf, nc2 = nc * nc, nc3 = nc2 * nc;
  __shared__ T Ps[2 * nf * nc];  // [child][nf][nc]
  __shared__ T u[G * nc3];       // [G][nc3]
  __shared__ T t1[G * nc2 * nf];  // [G][c2][c1][i0]
  __shared__ T t2[G * nc * nf2];  // [G][c2][i1][i0]
  __shared__ int chs[G];          // child position bits per cell
  const int tid = threadIdx.x, nt = blockDim.x;
  const long long cell0 = (long long)blockIdx.x * G;
  const int ncell = (int)min((long long)G, n_cells - cell0);
  for (int e = tid; e < 2 * nf * nc; e += nt) Ps[e] = (T)P.P[e / (nf * nc)][e % (nf * nc)];
  for (int lc = tid; lc < ncell; lc += nt) {
    long long cf = cell0 + lc;
    int code = 0;
    if (P.is_h) {
      int cx = (int)(cf % P.Nf[0]), cy = (int)((cf / P.Nf[0]) % P.Nf[1]),
          cz = (int)(cf / ((long long)P.Nf[0] * P.Nf[1]));
      code = (cx & 1) | ((cy & 1) << 1) | ((cz & 1) << 2);
    }
    chs[lc] = code;
  }
  for (int e = tid; e < ncell * nc3; e += nt) {
    int lc = e / nc3, j = e - lc * nc3;
    long long cf = cell0 + lc, cc = cf;
    if (P.is_h) {
      int cx = (int)(cf % P.Nf[0]), cy = (int)((cf / P.Nf[0]) % P.Nf[1]),
          cz = (int)(cf / ((long long)P.Nf[0] * P.Nf[1]));
      cc = (cx >> 1) + (long long)P.Nc[0] * ((cy >> 1) + (long long)P.Nc[1] * (cz >> 1));
    }
    u[e] = coarse[cc * nc3 + j];
  }
  __syncthreads();
  for (int e = tid; e < ncell * nc2 * nf; e += nt) {  // x
    int lc = e / (nc2 * nf), r = e - lc * nc2 * nf, i0 = r % nf, c21 = r / nf;
    const T* Pm = Ps + (chs[lc] & 1) * nf * nc + i0 * nc;
    const T* ul = u + lc * nc3 + c21 * nc;
    T acc = 0;
#pragma unroll
    for (int c = 0; c < nc; ++c) acc += Pm[c] * ul[c];
    t1[e] = acc;
  }
  __syncthreads();
  for (int e = tid; e < ncell * nc * nf2; e += nt) {  // y
    int lc = e / (nc * nf2), r = e - lc * nc * nf2, i0 = r % nf, i1 = (r / nf) % nf, c2 = r / nf2;
    const T* Pm = Ps + ((chs[lc] >> 1) & 1) * nf * nc + i1 * nc;
    const T* tl = t1 + lc * nc2 * nf + c2 * nc * nf + i0;
    T acc = 0;
#pragma unroll
    for (int c = 0; c < nc; ++c) acc += Pm[c] * tl[c * nf];
    t2[e] = acc;
  }
  __syncthreads();
  for (int e = tid; e < ncell * nf3; e += nt) {  // z, accumulate into the fine vector
    int lc = e / nf3, r = e - lc * nf3, i01 = r % nf2, i2 = r / nf2;
    const T* Pm = Ps + ((chs[lc] >> 2) & 1) * nf * nc + i2 * nc;
    const T* tl = t2 + lc * nc * nf2 + i01;
    T acc = 0;
#pragma unroll
    for (int c = 0; c < nc; ++c) acc += Pm[c] * tl[c * nf2];
    fine[cell0 * nf3 + e] += acc;
  }
}

template <int NF, int NC, int G, class T>
__global__ void __launch_bounds__(256) restrict_kernel(const __grid_constant__ TransferParams P,
                                                       const T* __restrict__ fine, T* __restrict__ coarse,
                                                       long long n_cells) {
  constexpr int nf = NF, nc = NC, nf2 = nf * nf, nf3 = nf2 * nf, nc2 = nc * nc, nc3 = nc2 * nc;
  __shared__ T Ps[2 * nf * nc];    // [child][nf][nc]
  __shared__ T f[G * nf3];         // [G][nf3]
  __shared__ T t1[G * nf2 * nc];   // [G][i2][i1][j0]
  __shared__ T t2[G * nf * nc2];   // [G][i2][j1][j0]
  __shared__ T acc[G * nc3];       // [G][nc3]
  const int tid = threadIdx.x, nt = blockDim.x;
  const long long cell0 = (long long)blockIdx.x * G;
  const int ncell = (int)min((long long)G, n_cells - cell0);
  for (int e = tid; e < 2 * nf * nc; e += nt) Ps[e] = (T)P.P[e / (nf * nc)][e % (nf * nc)];
  for (int e = tid; e < ncell * nc3; e += nt) acc[e] = 0;
  const int nch = P.is_h ? 8 : 1;
  for (int c8 = 0; c8 < nch; ++c8) {
    const int ch0 = c8 & 1, ch1 = (c8 >> 1) & 1, ch2 = (c8 >> 2) & 1;
    for (int e = tid; e < ncell * nf3; e += nt) {
      int lc = e / nf3, i = e - lc * nf3;
      long long cc = cell0 + lc, cf = cc;
      if (P.is_h) {
        int cx = (int)(cc % P.Nc[0]), cy = (int)((cc / P.Nc[0]) % P.Nc[1]),
            cz = (int)(cc / ((long long)P.Nc[0] * P.Nc[1]));
        cf = (2 * cx + ch0) + (long long)P.Nf[0] * ((2 * cy + ch1) + (long long)P.Nf[1] * (2 * cz + ch2));
      }
      f[e] = fine[cf * nf3 + i];
    }
    __syncthreads();
    const T* P0 = Ps + (P.is_h ? ch0 : 0) * nf * nc;
    const T* P1 = Ps + (P.is_h ? ch1 : 0) * nf * nc;
    const T* P2 = Ps + (P.is_h ? ch2 : 0) * nf * nc;
    for (int e = tid; e < ncell * nf2 * nc; e += nt) {  // x^T
      int lc = e / (nf2 * nc), r = e - lc * nf2 * nc, j0 = r % nc, i21 = r / nc;
      const T* fl = f + lc * nf3 + i21 * nf;
      T a = 0;
#pragma unroll
      for (int i = 0; i < nf; ++i) a += P0[i * nc + j0] * fl[i];
      t1[e] = a;
    }
    __syncthreads();
    for (int e = tid; e < ncell * nf * nc2; e += nt) {  // y^T
      int lc = e / (nf * nc2), r = e - lc * nf * nc2, j0 = r % nc, j1 = (r / nc) % nc, i2 = r / nc2;
      const T* tl = t1 + lc * nf2 * nc + i2 * nf * nc + j0;
      T a = 0;
#pragma unroll
      for (int i = 0; i < nf; ++i) a += P1[i * nc + j1] * tl[i * nc];
      t2[e] = a;
    }
    __syncthreads();
    for (int e = tid; e < ncell * nc3; e += nt) {  // z^T, accumulated over the children
      int lc = e / nc3, r = e - lc * nc3, j01 = r % nc2, j2 = r / nc2;
      const T* tl = t2 + lc * nf * nc2 + j01;
      T a = 0;
#pragma unroll
      for (int i = 0; i < nf; ++i) a += P2[i * nc + j2] * tl[i * nc2];
      acc[e] += a;
    }
    __syncthreads();
  }
  for (int e = tid; e < ncell * nc3; e += nt) coarse[cell0 * nc3 + e] += acc[e];
}

// (nf, nc) pairs of the level sequence: h-transfers at k = 1 and the Bisect p-sequence k -> k/2
#define EXG_TRANSFER_PAIRS(X) X(2, 2) X(3, 2) X(4, 2) X(5, 3) X(6, 3) X(7, 4) X(8, 4) X(9, 5)

template <class T>
void prolongate_add(const TransferParams& P, const T* coarse, T* fine, cudaStream_t s) {
  long long cells = (long long)P.Nf[0] * P.Nf[1] * P.Nf[2];
#define EXG_PROLONG(NF, NC)                                                                        \
  if (P.nf == NF && P.nc == NC) {                                                                  \
    using S = TransferShape<NF, NC, T>;                                                            \
    if (S::use_large(cells))                                                                       \
      prolongate_kernel<NF, NC, S::large, T>                                                       \
          <<<(unsigned)((cells + S::large - 1) / S::large), 256, 0, s>>>(P, coarse, fine, cells);  \
    else                                                                                           \
      prolongate_kernel<NF, NC, S::small, T>                                                       \
          <<<(unsigned)((cells + S::small - 1) / S::small), 256, 0, s>>>(P, coarse, fine, cells);  \
    EXG_CUDA(cudaGetLastError());                                                                  \
    return;                                                                                        \
  }
  EXG_TRANSFER_PAIRS(EXG_PROLONG)
#undef EXG_PROLONG
  throw Error{EXG_ERR_UNSUPPORTED, "unsupported transfer degree pair"};
}
template <class T>
void restrict_add(const TransferParams& P, const T* fine, T* coarse, cudaStream_t s) {
  long long cells = (long long)P.Nc[0] * P.Nc[1] * P.Nc[2];
#define EXG_RESTRICT(NF, NC)                                                                       \
  if (P.nf == NF && P.nc == NC) {                                                                  \
    using S = TransferShape<NF, NC, T>;                                                            \
    if (S::use_large(cells))                                                                       \
      restrict_kernel<NF, NC, S::large, T>                                                         \
          <<<(unsigned)((cells + S::large - 1) / S::large), 256, 0, s>>>(P, fine, coarse, cells);  \
    else                                                                                           \
      restrict_kernel<NF, NC, S::small, T>                                                         \
          <<<(unsigned)((cells + S::small - 1) / S::small), 256, 0, s>>>(P, fine, coarse, cells);  \
    EXG_CUDA(cudaGetLastError());                                                                  \
    return;                                                                                        \
  }
  EXG_TRANSFER_PAIRS(EXG_RESTRICT)
#undef EXG_RESTRICT
  throw Error{EXG_ERR_UNSUPPORTED, "unsupported transfer degree pair"};
}

// ------------------------------------------------------------------------------------------------
// coarse CG + point Jacobi in one CTA (MGCoarseKrylov, coarse_grid_solvers.h:157-224).  The dense
// coarse matrix is assembled at setup.  Iterations are bounded by max_iter.
// ------------------------------------------------------------------------------------------------
// block sum in FP64, valid in all threads; sh holds 33 values.  FP64 arithmetic runs at a small
// fraction of the FP32 rate on this part, so the partial sums are combined by warp 0 alone (one
// shuffle tree per warp, one for the warp partials) rather than redundantly by every thread.
__device__ __forceinline__ double cta_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = l < nw ? sh[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (l == 0) sh[32] = t;
  }
  __syncthreads();
  return sh[32];
}

// two block sums in the coarse precision, valid in all threads; sh holds 66 values
template <class R>
__device__ __forceinline__ void cta_sum2(R& a, R& b, R* sh) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) {
    sh[w] = a;
    sh[32 + w] = b;
  }
  __syncthreads();
  if (w == 0) {
    R ta = l < nw ? sh[l] : R(0), tb = l < nw ? sh[32 + l] : R(0);
    for (int o = 16; o > 0; o >>= 1) {
      ta += __shfl_down_sync(0xffffffffu, ta, o);
      tb += __shfl_down_sync(0xffffffffu, tb, o);
    }
    if (l == 0) {
      sh[64] = ta;
      sh[65] = tb;
    }
  }
  __syncthreads();
  a = sh[64];
  b = sh[65];
}

// out = A in with one thread per row.  The matrix is stored by columns (A[j*n + i] = A_ij, column j
// being the operator applied to e_j), so the threads of a warp read consecutive addresses
// (conflict-free in shared memory, coalesced in global memory); four partial sums per thread give
// independent FMA chains.  The summation order is fixed, so results are deterministic.
template <class CT>
__device__ __forceinline__ void coarse_matvec(const CT* A, const CT* in, CT* out, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    CT a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    int j = 0;
    for (; j + 3 < n; j += 4) {
      a0 += A[(long long)j * n + i] * in[j];
      a1 += A[(long long)(j + 1) * n + i] * in[j + 1];
      a2 += A[(long long)(j + 2) * n + i] * in[j + 2];
      a3 += A[(long long)(j + 3) * n + i] * in[j + 3];
    }
    for (; j < n; ++j) a0 += A[(long long)j * n + i] * in[j];
    out[i] = (a0 + a1) + (a2 + a3);
  }
  __syncthreads();
}

template <class T, class CT>
__global__ void __launch_bounds__(1024) coarse_cg_kernel(const CT* __restrict__ A, const CT* __restrict__ invd,
                                                         const T* __restrict__ rhs, T* __restrict__ xout,
                                                         CT* __restrict__ xstate, int n, double rel_tol,
                                                         double abs_tol, int max_iter, int singular, int stage_matrix,
                                                         long long* __restrict__ its_counter) {
  extern __shared__ __align__(16) unsigned char sm[];
  CT* x = reinterpret_cast<CT*>(sm);
  CT* r = x + n;
  CT* z = r + n;
  CT* p = z + n;
  CT* v = p + n;
  CT* As = v + n;  // n*n copy of the matrix when it fits in shared memory
  __shared__ double sh[33];
  __shared__ CT shc[66];
  __shared__ int s_nonzero;
  const int tid = threadIdx.x, nt = blockDim.x;
  const CT* Am = A;
  if (stage_matrix) {
    for (long long e = tid; e < (long long)n * n; e += nt) As[e] = A[e];
    Am = As;
  }
  if (tid == 0) s_nonzero = 0;
  // r = src (mean removed if singular)
  double mean = 0;
  if (singular) {
    double s = 0;
    for (int i = tid; i < n; i += nt) s += (double)rhs[i];
    mean = cta_sum(s, sh) / n;
  }
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    x[i] = xstate[i];
    z[i] = (CT)((double)rhs[i] - mean);  // b
    if (x[i] != CT(0)) s_nonzero = 1;
  }
  __syncthreads();
  // r = b - A x
  if (s_nonzero) {
    coarse_matvec(Am, x, v, n);
  } else {
    for (int i = tid; i < n; i += nt) v[i] = 0;
    __syncthreads();
  }
  // scalars in the coarse precision CT (deal.II's SolverCG on float vectors reduces in float);
  // z = D^-1 r is formed with the residual update so that r.r and r.z share one block reduction
  CT rr = 0, rz = 0;
  for (int i = tid; i < n; i += nt) {
    const CT ri = z[i] - v[i];
    const CT zi = invd[i] * ri;
    r[i] = ri;
    z[i] = zi;
    rr += ri * ri;
    rz += ri * zi;
  }
  cta_sum2(rr, rz, shc);
  CT rn = sqrt(rr);
  const CT tol = (CT)fmax(abs_tol, rel_tol * (double)rn);
  int it = 0;
  CT rho = rz, beta = 0;
  while (rn > tol && it < max_iter) {
    ++it;
    for (int i = tid; i < n; i += nt) p[i] = it == 1 ? z[i] : z[i] + beta * p[i];
    __syncthreads();
    coarse_matvec(Am, p, v, n);
    CT pv = 0, unused = 0;
    for (int i = tid; i < n; i += nt) pv += p[i] * v[i];
    cta_sum2(pv, unused, shc);
    const CT alpha = rho / pv;
    CT rr2 = 0, rz2 = 0;
    for (int i = tid; i < n; i += nt) {
      x[i] += alpha * p[i];
      const CT ri = r[i] - alpha * v[i];
      const CT zi = invd[i] * ri;
      r[i] = ri;
      z[i] = zi;
      rr2 += ri * ri;
      rz2 += ri * zi;
    }
    cta_sum2(rr2, rz2, shc);
    rn = sqrt(rr2);
    beta = rz2 / rho;
    rho = rz2;
  }
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    xstate[i] = x[i];
    xout[i] = (T)x[i];
  }
  if (tid == 0) its_counter[0] += it;
}

// raises the kernel's shared-memory limit for n unknowns (idempotent; call outside stream capture)
template <class T, class CT>
void coarse_cg_prepare(int n) {
  size_t vec_bytes = 5 * (size_t)n * sizeof(CT), mat_bytes = (size_t)n * n * sizeof(CT);
  size_t smem = vec_bytes + (vec_bytes + mat_bytes <= 200 * 1024 ? mat_bytes : 0);
  ensure_smem_attr((const void*)coarse_cg_kernel<T, CT>, (int)smem);
}

template <class T, class CT>
void coarse_cg(const CT* A, const CT* invd, const T* rhs, T* x, CT* xstate, int n, double rel_tol, double abs_tol,
               int max_iter, int singular, long long* its, cudaStream_t s) {
  size_t vec_bytes = 5 * (size_t)n * sizeof(CT), mat_bytes = (size_t)n * n * sizeof(CT);
  const int stage = vec_bytes + mat_bytes <= 200 * 1024 ? 1 : 0;
  size_t smem = vec_bytes + (stage ? mat_bytes : 0);
  auto k = coarse_cg_kernel<T, CT>;
  coarse_cg_prepare<T, CT>(n);
  // one thread per unknown (whole warps, at most 1024): idle threads would only add FP64 work to
  // every block reduction
  const int threads = std::min(1024, std::max(32, (n + 31) / 32 * 32));
  k<<<1, threads, smem, s>>>(A, invd, rhs, x, xstate, n, rel_tol, abs_tol, max_iter, singular, stage, its);
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
template void coarse_cg_prepare<float, float>(int);
template void coarse_cg_prepare<float, double>(int);
template void coarse_cg_prepare<double, double>(int);
template void coarse_cg<float, double>(const double*, const double*, const float*, float*, double*, int, double,
                                       double, int, int, long long*, cudaStream_t);
template void coarse_cg<double, double>(const double*, const double*, const double*, double*, double*, int, double,
                                        double, int, int, long long*, cudaStream_t);

}  // namespace exg
