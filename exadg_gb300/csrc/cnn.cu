// Cell-patch convolutional network for the learned initial guess of the pressure-Poisson sequence.
//
// Network (FP32, channel-major activations [C][n_cells] on a periodic structured cell grid):
//   h1 = SiLU(W1 * x + b1)            1x1x1, c_in  -> c_hid
//   h2 = SiLU(W2 (*) h1 + b2)         3x3x3 periodic, c_hid -> c_hid
//   y  =       W3 (*) h2 + b3         3x3x3 periodic, c_hid -> c_out
// The input x holds, per cell, the DG coefficients of the last pressures and of the current
// right-hand side; y is the correction added to the polynomial extrapolation of the pressure.
// Forward, backward (data and weight gradients) and the Adam update are hand-written kernels;
// the weight-gradient reduction is deterministic (per-chunk partials summed in index order).
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "cnn.h"
#include "internal.h"

namespace exg {

static constexpr int CNN_MAX_C = 32;

__device__ __forceinline__ int wrap(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

template <int K>
__device__ __forceinline__ int tap_neighbor(int x, int y, int z, int t, int nx, int ny, int nz) {
  if (K == 1) return x + nx * (y + ny * z);
  int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
  return wrap(x + dx, nx) + nx * (wrap(y + dy, ny) + ny * wrap(z + dz, nz));
}

__device__ __forceinline__ float silu(float v) { return v / (1.0f + __expf(-v)); }
__device__ __forceinline__ float silu_grad(float v) {
  float s = 1.0f / (1.0f + __expf(-v));
  return s * (1.0f + v * (1.0f - s));
}

// out[co][c] = act(bias[co] + sum_{ci,t} W[co][ci][t] in[ci][nb(c,t)]); pre keeps the
// pre-activation for the backward pass.  W layout [co][ci][t].  A thread owns one cell and a group
// of CONV_CG output channels (blockIdx.y selects the group), so a launch has ceil(cout / CONV_CG)
// times as many threads as cells.  The group's weights are staged in shared memory per chunk of
// input channels as [ci][t][co], so two float4 reads serve the eight channels of a tap.
static constexpr int CONV_CG = 8;
static constexpr int CONV_CI_CHUNK = 16;

template <int K>
__global__ void __launch_bounds__(128) conv_fwd_kernel(const float* __restrict__ in, const float* __restrict__ W,
                                                       const float* __restrict__ bias, float* __restrict__ out,
                                                       float* __restrict__ pre, int cin, int cout, int nx, int ny,
                                                       int nz, int act, int accumulate) {
  constexpr int K3 = K * K * K;
  __shared__ __align__(16) float sW[CONV_CI_CHUNK * K3 * CONV_CG];
  const int nc = nx * ny * nz;
  const int co0 = blockIdx.y * CONV_CG;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const bool ok = c < nc;
  int x = 0, y = 0, z = 0;
  if (ok) {
    x = c % nx;
    y = (c / nx) % ny;
    z = c / (nx * ny);
  }
  int nbr[K3];
#pragma unroll
  for (int t = 0; t < K3; ++t) nbr[t] = tap_neighbor<K>(x, y, z, t, nx, ny, nz);
  float acc[CONV_CG];
#pragma unroll
  for (int q = 0; q < CONV_CG; ++q) acc[q] = (co0 + q < cout && bias) ? bias[co0 + q] : 0.0f;
  for (int ci0 = 0; ci0 < cin; ci0 += CONV_CI_CHUNK) {
    const int nci = min(CONV_CI_CHUNK, cin - ci0);
    __syncthreads();
    for (int i = threadIdx.x; i < CONV_CI_CHUNK * K3 * CONV_CG; i += blockDim.x) {
      int q = i % CONV_CG, t = (i / CONV_CG) % K3, cil = i / (CONV_CG * K3);
      int co = co0 + q;
      sW[i] = (co < cout && cil < nci) ? W[((size_t)co * cin + ci0 + cil) * K3 + t] : 0.0f;
    }
    __syncthreads();
    if (ok) {
      for (int cil = 0; cil < nci; ++cil) {
        const float* src = in + (size_t)(ci0 + cil) * nc;
        const float4* w4 = reinterpret_cast<const float4*>(sW + cil * K3 * CONV_CG);
#pragma unroll
        for (int t = 0; t < K3; ++t) {
          const float v = __ldg(src + nbr[t]);
          const float4 wa = w4[2 * t], wb = w4[2 * t + 1];
          acc[0] = fmaf(wa.x, v, acc[0]);
          acc[1] = fmaf(wa.y, v, acc[1]);
          acc[2] = fmaf(wa.z, v, acc[2]);
          acc[3] = fmaf(wa.w, v, acc[3]);
          acc[4] = fmaf(wb.x, v, acc[4]);
          acc[5] = fmaf(wb.y, v, acc[5]);
          acc[6] = fmaf(wb.z, v, acc[6]);
          acc[7] = fmaf(wb.w, v, acc[7]);
        }
      }
    }
  }
  if (ok) {
#pragma unroll
    for (int q = 0; q < CONV_CG; ++q) {
      const int co = co0 + q;
      if (co >= cout) break;
      if (pre) pre[(size_t)co * nc + c] = acc[q];
      float r = act ? silu(acc[q]) : acc[q];
      if (accumulate) r += out[(size_t)co * nc + c];
      out[(size_t)co * nc + c] = r;
    }
  }
}

// g_pre = g_post * SiLU'(pre), in place on g
__global__ void silu_backward_kernel(float* __restrict__ g, const float* __restrict__ pre, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    g[i] *= silu_grad(pre[i]);
}

// W^T with flipped taps: Wt[ci][co][t'] = W[co][ci][K3-1-t'] (transposed convolution = backward data)
__global__ void transpose_flip_kernel(const float* __restrict__ W, float* __restrict__ Wt, int cout, int cin, int k3) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cout * cin * k3) return;
  int t = i % k3, ci = (i / k3) % cin, co = i / (k3 * cin);
  Wt[((size_t)ci * cout + co) * k3 + (k3 - 1 - t)] = W[i];
}

// partial weight gradients per chunk of CHUNK cells:
//   gWp[chunk][co][ci][t] = sum_{c in chunk} gout[co][c] in[ci][nb(c,t)],  gbp[chunk][co] = sum gout[co][c]
template <int K>
__global__ void conv_wgrad_kernel(const float* __restrict__ in, const float* __restrict__ gout,
                                  float* __restrict__ gWp, float* __restrict__ gbp, int cin, int cout, int nx, int ny,
                                  int nz, int chunk) {
  constexpr int K3 = K * K * K;
  extern __shared__ __align__(16) float sm[];
  // rows padded to chunk + 1 floats: the threads of a warp read column l of different rows
  const int cs = chunk + 1;
  float* sg = sm;                // [cout][cs]
  float* sx = sm + cout * cs;    // [K3][cs] for one input channel
  const int nc = nx * ny * nz;
  const int ch = blockIdx.x, ci = blockIdx.y;
  const int c0 = ch * chunk;
  const int ncl = min(chunk, nc - c0);
  for (int i = threadIdx.x; i < cout * chunk; i += blockDim.x) {
    int co = i / chunk, l = i % chunk;
    sg[co * cs + l] = l < ncl ? gout[(size_t)co * nc + c0 + l] : 0.0f;
  }
  for (int i = threadIdx.x; i < K3 * chunk; i += blockDim.x) {
    int t = i / chunk, l = i % chunk;
    float v = 0.0f;
    if (l < ncl) {
      int c = c0 + l, x = c % nx, y = (c / nx) % ny, z = c / (nx * ny);
      v = in[(size_t)ci * nc + tap_neighbor<K>(x, y, z, t, nx, ny, nz)];
    }
    sx[t * cs + l] = v;
  }
  __syncthreads();
  for (int pidx = threadIdx.x; pidx < cout * K3; pidx += blockDim.x) {
    int co = pidx / K3, t = pidx % K3;
    const float* g = sg + co * cs;
    const float* xv = sx + t * cs;
    float s = 0.0f;
    for (int l = 0; l < chunk; ++l) s = fmaf(g[l], xv[l], s);
    gWp[(((size_t)ch * cout + co) * cin + ci) * K3 + t] = s;
  }
  if (ci == 0)
    for (int co = threadIdx.x; co < cout; co += blockDim.x) {
      const float* g = sg + co * cs;
      float s = 0.0f;
      for (int l = 0; l < chunk; ++l) s += g[l];
      gbp[(size_t)ch * cout + co] = s;
    }
}

// out[i] = sum_ch part[ch][i], fixed order
__global__ void chunk_sum_kernel(const float* __restrict__ part, float* __restrict__ out, long long n, int nch) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int ch = 0; ch < nch; ++ch) s += part[(size_t)ch * n + i];
  out[i] = s;
}

// loss = mean (y - t)^2 over all entries, gy = 2 (y - t) / n ; per-block partial losses
__global__ void mse_kernel(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ gy,
                           float* __restrict__ partial, long long n) {
  __shared__ float sh[32];
  float s = 0.0f;
  const float inv = 1.0f / (float)n;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float d = y[i] - t[i];
    gy[i] = 2.0f * d * inv;
    s += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float r = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += sh[w];
    partial[blockIdx.x] = r * inv;
  }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                            float c2, float scale) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gi = g[i] * scale;
  float mi = b1 * m[i] + (1.0f - b1) * gi;
  float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void axpy_f32_kernel(float* __restrict__ y, const float* __restrict__ x, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += x[i];
}

// ---------------------------------------------------------------------------------------------------
// DG vector <-> network tensor
// ---------------------------------------------------------------------------------------------------
// x[j*npc + i][c] = vec_j[c*npc + i] * inv_scale_j  (j-th of nvec FP64 DG vectors, npc DoF per cell)
__global__ void pack_kernel(const double* const* __restrict__ vecs, const double* __restrict__ inv_scale, int nvec,
                            int npc, long long n_cells, float* __restrict__ x) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long tot = (long long)nvec * npc * n_cells;
  if (g >= tot) return;
  long long c = g % n_cells;
  long long ch = g / n_cells;
  int j = (int)(ch / npc), i = (int)(ch % npc);
  x[g] = (float)(vecs[j][c * npc + i] * inv_scale[j]);
}

// dst[c*npc + i] = base[c*npc + i] + scale * y[i][c]
__global__ void unpack_add_kernel(const float* __restrict__ y, const double* __restrict__ base, double scale, int npc,
                                  long long n_cells, double* __restrict__ dst) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_cells * npc) return;
  long long c = g / npc;
  int i = (int)(g % npc);
  dst[g] = base[g] + scale * (double)y[(size_t)i * n_cells + c];
}

// t[i][c] = (a[c*npc+i] - b[c*npc+i]) * inv_scale
__global__ void pack_diff_kernel(const double* __restrict__ a, const double* __restrict__ b, double inv_scale, int npc,
                                 long long n_cells, float* __restrict__ t) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_cells * npc) return;
  long long i = g / n_cells, c = g % n_cells;
  t[g] = (float)((a[c * npc + i] - b[c * npc + i]) * inv_scale);
}

// ---------------------------------------------------------------------------------------------------
// guess assembly without host round trips: feature scaling and the least-squares step length are
// reduced on the device (per-block partials in a static array, summed in index order by one warp per
// quantity).  Calls that overlap on the GPU share the partials array and race.
// ---------------------------------------------------------------------------------------------------
static constexpr int RED_NB = 608;  // 4 blocks per SM
__device__ double g_dg_partials[6 * RED_NB];

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// partials[j][block] = the block's part of sum_i q_j(i):
//   KIND 0 (features, a = p0, b = p1, c = p2, d = r): p0^2, d1^2, d2^2, r^2
//   KIND 1 (least squares, a = r, b = Ae, c = Af or null): r.Ae, Ae.Ae, r.r, r.Af, Af.Af, Ae.Af
template <int KIND>
__global__ void __launch_bounds__(256) dg_partials_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                                          const double* __restrict__ c, const double* __restrict__ d,
                                                          long long n) {
  constexpr int NF = KIND == 0 ? 4 : 6;
  double acc[NF];
#pragma unroll
  for (int j = 0; j < NF; ++j) acc[j] = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if constexpr (KIND == 0) {
      const double p0 = a[i], p1 = b[i], p2 = c[i], rr = d[i];
      const double d1 = p0 - p1, d2 = p0 - 2.0 * p1 + p2;
      acc[0] += p0 * p0;
      acc[1] += d1 * d1;
      acc[2] += d2 * d2;
      acc[3] += rr * rr;
    } else {
      const double r = a[i], ae = b[i];
      acc[0] += r * ae;
      acc[1] += ae * ae;
      acc[2] += r * r;
      if (c) {
        const double af = c[i];
        acc[3] += r * af;
        acc[4] += af * af;
        acc[5] += ae * af;
      }
    }
  }
  __shared__ double sh[NF][8];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < NF; ++j) {
    double v = warp_sum_d(acc[j]);
    if (l == 0) sh[j][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < NF) {
    double v = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) v += sh[threadIdx.x][k];
    g_dg_partials[threadIdx.x * RED_NB + blockIdx.x] = v;
  }
}

// one warp per quantity sums the partials in index order, then
//   mode 0: out[0..3] = RMS of the features; out[2] = diff_scale if diff_scale > 0
//   mode 1: least-squares step lengths along e (and f), see exg_dg_ls_step
__global__ void dg_finalize_kernel(int nq, int mode, long long n, double diff_scale, double* __restrict__ out) {
  __shared__ double tot[6];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (w < nq) {
    double v = 0.0;
    for (int k = l; k < RED_NB; k += 32) v += g_dg_partials[w * RED_NB + k];
    v = warp_sum_d(v);
    if (l == 0) tot[w] = v;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  if (mode == 0) {
    for (int j = 0; j < 4; ++j) out[j] = fmax(sqrt(tot[j] / (double)n), 1e-300);
    if (diff_scale > 0.0) out[2] = diff_scale;
    return;
  }
  // minimise |r - ce Ae - cf Af|: normal equations [[Ae.Ae, Ae.Af], [Ae.Af, Af.Af]] (ce, cf) = (r.Ae, r.Af)
  const double rae = tot[0], aa = tot[1], rr = tot[2];
  double ce = aa > 0.0 ? rae / aa : 0.0, cf = 0.0;
  if (nq == 6) {
    const double raf = tot[3], ff = tot[4], af = tot[5];
    const double det = aa * ff - af * af;
    if (det > 1e-12 * aa * ff && aa > 0.0 && ff > 0.0) {
      ce = (rae * ff - raf * af) / det;
      cf = (raf * aa - rae * af) / det;
    } else if (ff > 0.0 && raf * raf / ff > rae * rae / fmax(aa, 1e-300)) {
      ce = 0.0;  // (nearly) parallel directions: the better single one
      cf = raf / ff;
    }
  }
  if (!isfinite(ce) || !isfinite(cf)) ce = cf = 0.0;
  double red = ce * rae + cf * (nq == 6 ? tot[3] : 0.0);  // |r|^2 - |r - ce Ae - cf Af|^2
  if (!(red > 1e-14 * rr)) ce = cf = 0.0;  // no decrease beyond rounding: plain base (fallback)
  out[0] = rae;
  out[1] = aa;
  out[2] = rr;
  out[3] = ce;
  out[4] = cf;
  out[5] = ce == 0.0 && cf == 0.0 ? 0.0 : red;
}

// x[j*npc + i][c] = f_j[c*npc + i] / rms_j with f = (p0, p0 - p1, p0 - 2 p1 + p2, r)
__global__ void dg_features_pack_kernel(const double* __restrict__ p0, const double* __restrict__ p1,
                                        const double* __restrict__ p2, const double* __restrict__ r,
                                        const double* __restrict__ rms, int npc, long long n_cells,
                                        float* __restrict__ x) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= 4LL * npc * n_cells) return;
  long long c = g % n_cells;
  long long ch = g / n_cells;
  int j = (int)(ch / npc), i = (int)(ch % npc);
  long long k = c * npc + i;
  double v;
  if (j == 0)
    v = p0[k];
  else if (j == 1)
    v = p0[k] - p1[k];
  else if (j == 2)
    v = p0[k] - 2.0 * p1[k] + p2[k];
  else
    v = r[k];
  x[g] = (float)(v / rms[j]);
}

// x = base + stats[3] e + stats[4] f (f optional)
__global__ void dg_step_kernel(const double* __restrict__ base, const double* __restrict__ e,
                               const double* __restrict__ f, const double* __restrict__ stats, long long n,
                               double* __restrict__ x) {
  const double ce = stats[3], cf = stats[4];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = base[i] + ce * e[i] + (f ? cf * f[i] : 0.0);
}

// ---------------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------------
static void* cnn_alloc(size_t bytes) {
  void* p = nullptr;
  EXG_CUDA(cudaMalloc(&p, bytes));
  EXG_CUDA(cudaMemset(p, 0, bytes));
  return p;
}

static void conv_fwd(int K, int cout, const float* in, const float* W, const float* b, float* out, float* pre,
                     int cin, const int N[3], int act, cudaStream_t s, int acc = 0) {
  EXG_CHECK(cout >= 1 && cout <= CNN_MAX_C, EXG_ERR_UNSUPPORTED, "conv: at most 32 output channels");
  int nc = N[0] * N[1] * N[2];
  dim3 grid((unsigned)((nc + 127) / 128), (unsigned)((cout + CONV_CG - 1) / CONV_CG));
  if (K == 1)
    conv_fwd_kernel<1><<<grid, 128, 0, s>>>(in, W, b, out, pre, cin, cout, N[0], N[1], N[2], act, acc);
  else
    conv_fwd_kernel<3><<<grid, 128, 0, s>>>(in, W, b, out, pre, cin, cout, N[0], N[1], N[2], act, acc);
  EXG_CUDA(cudaGetLastError());
}

}  // namespace exg

using namespace exg;

// the conv kernels write only channels < COUT; the template width covers cout
static void check_width(int K, int c) {
  (void)K;
  EXG_CHECK(c <= 32, EXG_ERR_UNSUPPORTED, "at most 32 channels per layer");
}

exg_cnn::exg_cnn(const int n[3], int cin, int chid, int cout, unsigned long long seed)
    : c_in(cin), c_hid(chid), c_out(cout) {
  EXG_CHECK(cin >= 1 && chid >= 1 && chid <= 32 && cout >= 1 && cout <= 32, EXG_ERR_UNSUPPORTED,
            "cnn: 1 <= hidden, out channels <= 32");
  for (int e = 0; e < 3; ++e) {
    EXG_CHECK(n[e] >= 1, EXG_ERR_INVALID, "cnn: grid size");
    N[e] = n[e];
  }
  check_width(1, chid);
  check_width(3, cout);
  n_cells = (long long)N[0] * N[1] * N[2];
  off[0] = 0;                               // W1 [chid][cin]
  off[1] = off[0] + (long long)chid * cin;  // b1
  off[2] = off[1] + chid;                   // W2 [chid][chid][27]
  off[3] = off[2] + (long long)chid * chid * 27;  // b2
  off[4] = off[3] + chid;                   // W3 [cout][chid][27]
  off[5] = off[4] + (long long)cout * chid * 27;  // b3
  off[6] = off[5] + cout;                          // W4 [cout][cin], linear skip x -> y
  n_params = off[6] + (long long)cout * cin;
  params = (float*)cnn_alloc(n_params * 4);
  grads = (float*)cnn_alloc(n_params * 4);
  m = (float*)cnn_alloc(n_params * 4);
  v = (float*)cnn_alloc(n_params * 4);
  // He-style initialisation with a splitmix64 generator (host), biases zero
  std::vector<float> h(n_params, 0.0f);
  unsigned long long st = seed;
  auto next = [&]() {
    st += 0x9E3779B97F4A7C15ull;
    unsigned long long z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  auto fill = [&](long long o, long long cnt, double fan_in, double gain) {
    double a = gain * std::sqrt(3.0 / fan_in);
    for (long long i = 0; i < cnt; ++i) h[o + i] = (float)((2.0 * next() - 1.0) * a);
  };
  fill(off[0], off[1] - off[0], cin, 1.4);
  fill(off[2], off[3] - off[2], 27.0 * chid, 1.4);
  fill(off[4], off[5] - off[4], 27.0 * chid, 0.1);  // small output layer: starts close to extrapolation
  // W4 (skip) starts at zero
  EXG_CUDA(cudaMemcpy(params, h.data(), n_params * 4, cudaMemcpyHostToDevice));
  a1 = (float*)cnn_alloc(n_cells * chid * 4);
  p1 = (float*)cnn_alloc(n_cells * chid * 4);
  a2 = (float*)cnn_alloc(n_cells * chid * 4);
  p2 = (float*)cnn_alloc(n_cells * chid * 4);
  y = (float*)cnn_alloc(n_cells * cout * 4);
  g2 = (float*)cnn_alloc(n_cells * chid * 4);
  g1 = (float*)cnn_alloc(n_cells * chid * 4);
  gy = (float*)cnn_alloc(n_cells * cout * 4);
  wt = (float*)cnn_alloc((long long)32 * 32 * 27 * 4);
  chunk = 256;
  n_chunks = (int)((n_cells + chunk - 1) / chunk);
  long long maxw = std::max<long long>((long long)chid * cin, (long long)32 * 32 * 27);
  wpart = (float*)cnn_alloc((size_t)n_chunks * maxw * 4);
  bpart = (float*)cnn_alloc((size_t)n_chunks * 32 * 4);
  loss_part = (float*)cnn_alloc(1024 * 4);
  bskip = (float*)cnn_alloc(32 * 4);
  long long need = (long long)cout * cin;
  EXG_CHECK(need <= maxw, EXG_ERR_UNSUPPORTED, "cnn: skip layer larger than the gradient scratch");
}

exg_cnn::~exg_cnn() {
  for (float* p : {params, grads, m, v, a1, p1, a2, p2, y, g2, g1, gy, wt, wpart, bpart, loss_part, bskip})
    if (p) cudaFree(p);
}

void exg_cnn::forward(const float* x, float* out, bool keep, cudaStream_t s) {
  conv_fwd(1, c_hid, x, params + off[0], params + off[1], a1, keep ? p1 : nullptr, c_in, N, 1, s);
  conv_fwd(3, c_hid, a1, params + off[2], params + off[3], a2, keep ? p2 : nullptr, c_hid, N, 1, s);
  conv_fwd(3, c_out, a2, params + off[4], params + off[5], out ? out : y, nullptr, c_hid, N, 0, s);
  conv_fwd(1, c_out, x, params + off[6], nullptr, out ? out : y, nullptr, c_in, N, 0, s, 1);
}

void exg_cnn::wgrad(int K, const float* in, const float* g, int cin, int cout, float* gW, float* gb, cudaStream_t s) {
  int K3 = K * K * K;
  size_t smem = ((size_t)cout + K3) * (chunk + 1) * 4;
  ensure_smem_attr((const void*)conv_wgrad_kernel<3>, 64 * 1024);
  ensure_smem_attr((const void*)conv_wgrad_kernel<1>, 64 * 1024);
  EXG_CHECK(smem <= 64 * 1024, EXG_ERR_UNSUPPORTED, "cnn: weight-gradient tile too large");
  dim3 grid(n_chunks, cin);
  if (K == 1)
    conv_wgrad_kernel<1><<<grid, 256, smem, s>>>(in, g, wpart, bpart, cin, cout, N[0], N[1], N[2], chunk);
  else
    conv_wgrad_kernel<3><<<grid, 256, smem, s>>>(in, g, wpart, bpart, cin, cout, N[0], N[1], N[2], chunk);
  EXG_CUDA(cudaGetLastError());
  long long nw = (long long)cout * cin * K3;
  chunk_sum_kernel<<<(unsigned)((nw + 255) / 256), 256, 0, s>>>(wpart, gW, nw, n_chunks);
  chunk_sum_kernel<<<(unsigned)((cout + 255) / 256), 256, 0, s>>>(bpart, gb, cout, n_chunks);
  EXG_CUDA(cudaGetLastError());
}

void exg_cnn::backward(const float* x, const float* gout, cudaStream_t s) {
  // forward with stored pre-activations
  forward(x, nullptr, true, s);
  // layer 3: y = W3 (*) a2 + b3
  wgrad(3, a2, gout, c_hid, c_out, grads + off[4], grads + off[5], s);
  // g2 = W3^T (*) gout, then through SiLU
  {
    int tot = c_out * c_hid * 27;
    transpose_flip_kernel<<<(tot + 255) / 256, 256, 0, s>>>(params + off[4], wt, c_out, c_hid, 27);
    conv_fwd(3, c_hid, gout, wt, nullptr, g2, nullptr, c_out, N, 0, s);
    silu_backward_kernel<<<1024, 256, 0, s>>>(g2, p2, n_cells * c_hid);
  }
  // layer 2
  wgrad(3, a1, g2, c_hid, c_hid, grads + off[2], grads + off[3], s);
  {
    int tot = c_hid * c_hid * 27;
    transpose_flip_kernel<<<(tot + 255) / 256, 256, 0, s>>>(params + off[2], wt, c_hid, c_hid, 27);
    conv_fwd(3, c_hid, g2, wt, nullptr, g1, nullptr, c_hid, N, 0, s);
    silu_backward_kernel<<<1024, 256, 0, s>>>(g1, p1, n_cells * c_hid);
  }
  // layer 1 (1x1x1)
  wgrad(1, x, g1, c_in, c_hid, grads + off[0], grads + off[1], s);
  // linear skip: gW4 = gout x^T (its bias slot is scratch)
  wgrad(1, x, gout, c_in, c_out, grads + off[6], bskip, s);
  EXG_CUDA(cudaGetLastError());
}

float exg_cnn::loss_and_grad(const float* x, const float* target, cudaStream_t s) {
  forward(x, nullptr, false, s);
  long long n = n_cells * c_out;
  mse_kernel<<<256, 256, 0, s>>>(y, target, gy, loss_part, n);
  EXG_CUDA(cudaGetLastError());
  backward(x, gy, s);
  std::vector<float> lp(256);
  EXG_CUDA(cudaMemcpyAsync(lp.data(), loss_part, 256 * 4, cudaMemcpyDeviceToHost, s));
  EXG_CUDA(cudaStreamSynchronize(s));
  double l = 0;
  for (float f : lp) l += f;
  return (float)l;
}

void exg_cnn::adam(float lr, float grad_scale, cudaStream_t s) {
  ++step;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  float c1 = 1.0f - std::pow(b1, (float)step), c2 = 1.0f - std::pow(b2, (float)step);
  adam_kernel<<<(unsigned)((n_params + 255) / 256), 256, 0, s>>>(params, grads, m, v, n_params, lr, b1, b2, eps, c1,
                                                                  c2, grad_scale);
  EXG_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------------
#define CNN_BEGIN try {
#define CNN_END                   \
  }                               \
  catch (const exg::Error& e) {   \
    exg::set_error(e.msg);        \
    return e.status;              \
  }                               \
  catch (...) {                   \
    exg::set_error("cnn error");  \
    return EXG_ERR_INVALID;       \
  }                               \
  return EXG_OK;

extern "C" {

exg_status exg_cnn_create(const int n_cells[3], int c_in, int c_hidden, int c_out, unsigned long long seed,
                          exg_cnn** cnn) {
  CNN_BEGIN
  EXG_CHECK(n_cells && cnn, EXG_ERR_INVALID, "null argument");
  *cnn = new exg_cnn(n_cells, c_in, c_hidden, c_out, seed);
  CNN_END
}

exg_status exg_cnn_destroy(exg_cnn* cnn) {
  CNN_BEGIN
  delete cnn;
  CNN_END
}

exg_status exg_cnn_n_params(const exg_cnn* cnn, long long* n) {
  CNN_BEGIN
  EXG_CHECK(cnn && n, EXG_ERR_INVALID, "null argument");
  *n = cnn->n_params;
  CNN_END
}

exg_status exg_cnn_params(exg_cnn* cnn, float** params, float** grads) {
  CNN_BEGIN
  EXG_CHECK(cnn, EXG_ERR_INVALID, "null argument");
  if (params) *params = cnn->params;
  if (grads) *grads = cnn->grads;
  CNN_END
}

exg_status exg_cnn_forward(exg_cnn* cnn, const float* x, float* y, void* stream) {
  CNN_BEGIN
  EXG_CHECK(cnn && x && y, EXG_ERR_INVALID, "null argument");
  cnn->forward(x, y, false, (cudaStream_t)stream);
  CNN_END
}

exg_status exg_cnn_backward(exg_cnn* cnn, const float* x, const float* gy, void* stream) {
  CNN_BEGIN
  EXG_CHECK(cnn && x && gy, EXG_ERR_INVALID, "null argument");
  cnn->backward(x, gy, (cudaStream_t)stream);
  CNN_END
}

exg_status exg_cnn_train_step(exg_cnn* cnn, const float* x, const float* target, float lr, float* loss,
                              void* stream) {
  CNN_BEGIN
  EXG_CHECK(cnn && x && target, EXG_ERR_INVALID, "null argument");
  float l = cnn->loss_and_grad(x, target, (cudaStream_t)stream);
  cnn->adam(lr, 1.0f, (cudaStream_t)stream);
  if (loss) *loss = l;
  CNN_END
}

exg_status exg_cnn_optimizer_state(exg_cnn* cnn, float** m, float** v, long long** step) {
  CNN_BEGIN
  EXG_CHECK(cnn && m && v && step, EXG_ERR_INVALID, "null argument");
  *m = cnn->m;
  *v = cnn->v;
  *step = &cnn->step;
  CNN_END
}

exg_status exg_cnn_adam(exg_cnn* cnn, float lr, void* stream) {
  CNN_BEGIN
  EXG_CHECK(cnn, EXG_ERR_INVALID, "null argument");
  cnn->adam(lr, 1.0f, (cudaStream_t)stream);
  CNN_END
}

exg_status exg_dg_pack(const double* const* vecs, const double* inv_scales, int n_vec, int dofs_per_cell,
                       long long n_cells, float* x, void* stream) {
  CNN_BEGIN
  EXG_CHECK(vecs && inv_scales && x, EXG_ERR_INVALID, "null argument");
  long long tot = (long long)n_vec * dofs_per_cell * n_cells;
  pack_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, (cudaStream_t)stream>>>(vecs, inv_scales, n_vec, dofs_per_cell,
                                                                               n_cells, x);
  EXG_CUDA(cudaGetLastError());
  CNN_END
}

exg_status exg_dg_unpack_add(const float* y, const double* base, double scale, int dofs_per_cell, long long n_cells,
                             double* dst, void* stream) {
  CNN_BEGIN
  EXG_CHECK(y && base && dst, EXG_ERR_INVALID, "null argument");
  long long tot = n_cells * dofs_per_cell;
  unpack_add_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, (cudaStream_t)stream>>>(y, base, scale, dofs_per_cell,
                                                                                     n_cells, dst);
  EXG_CUDA(cudaGetLastError());
  CNN_END
}

exg_status exg_dg_pack_diff(const double* a, const double* b, double inv_scale, int dofs_per_cell, long long n_cells,
                            float* t, void* stream) {
  CNN_BEGIN
  EXG_CHECK(a && b && t, EXG_ERR_INVALID, "null argument");
  long long tot = n_cells * dofs_per_cell;
  pack_diff_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a, b, inv_scale, dofs_per_cell,
                                                                                    n_cells, t);
  EXG_CUDA(cudaGetLastError());
  CNN_END
}

exg_status exg_dg_features(const double* p0, const double* p1, const double* p2, const double* r,
                           int dofs_per_cell, long long n_cells, double diff_scale, float* x, double* rms,
                           void* stream) {
  CNN_BEGIN
  EXG_CHECK(p0 && p1 && p2 && r && x && rms, EXG_ERR_INVALID, "null argument");
  EXG_CHECK(dofs_per_cell >= 1 && n_cells >= 1, EXG_ERR_INVALID, "empty vectors");
  cudaStream_t s = (cudaStream_t)stream;
  const long long n = n_cells * dofs_per_cell;
  dg_partials_kernel<0><<<RED_NB, 256, 0, s>>>(p0, p1, p2, r, n);
  dg_finalize_kernel<<<1, 128, 0, s>>>(4, 0, n, diff_scale, rms);
  const long long tot = 4 * n;
  dg_features_pack_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(p0, p1, p2, r, rms, dofs_per_cell, n_cells,
                                                                        x);
  EXG_CUDA(cudaGetLastError());
  CNN_END
}

exg_status exg_dg_ls_step(const double* r, const double* Ae, const double* e, const double* Af, const double* f,
                          const double* base, long long n, double* x, double* stats, void* stream) {
  CNN_BEGIN
  EXG_CHECK(r && Ae && e && base && x && stats, EXG_ERR_INVALID, "null argument");
  EXG_CHECK((Af == nullptr) == (f == nullptr), EXG_ERR_INVALID, "give both f and A f, or neither");
  EXG_CHECK(n >= 1, EXG_ERR_INVALID, "empty vectors");
  cudaStream_t s = (cudaStream_t)stream;
  dg_partials_kernel<1><<<RED_NB, 256, 0, s>>>(r, Ae, Af, nullptr, n);
  dg_finalize_kernel<<<1, 192, 0, s>>>(f ? 6 : 3, 1, n, 0.0, stats);
  dg_step_kernel<<<RED_NB * 2, 256, 0, s>>>(base, e, f, stats, n, x);
  EXG_CUDA(cudaGetLastError());
  CNN_END
}

}  // extern "C"
