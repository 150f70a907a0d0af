// Continuous levels of cphMG on Cartesian meshes (declarations and the algorithm in lattice.h).
//
// Apply: one CTA per TX x TY x TZ tile of output nodes.  The tile and a halo of k nodes per side
// are read once into shared memory (constrained nodes and nodes outside a bounded lattice as
// zero, periodic directions wrapped), then three 1D band passes run in shared memory:
//   z: a = M_z x, b = K_z x            (a thread per (x, y) column, the column in registers)
//   y: c = M_y a, d = K_y a + M_y b    (a thread per (x, z) column; c, d reuse the input space)
//   x: A x = K_x c + M_x d             (a thread per output node, coalesced store through the
//                                       point epilogue; constrained nodes store src)
// Global traffic is one read of src (plus the halo, mostly from L2) and one write of dst.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "epilogue.cuh"
#include "lattice.h"

namespace exg {

LatticeHost::~LatticeHost() {
  if (coef_dev) cudaFree(coef_dev);
}

void make_lattice(const MeshInfo& m, int k, bool singular, LatticeHost& L) {
  EXG_CHECK(m.affine(), EXG_ERR_UNSUPPORTED, "continuous multigrid levels need a Cartesian mesh");
  EXG_CHECK(k >= 1 && k <= LAT_KMAX, EXG_ERR_UNSUPPORTED, "continuous level degree must be 1..8");
  L.k = k;
  for (int d = 0; d < 3; ++d) {
    L.N[d] = m.N[d];
    L.mask.periodic[d] = m.d.periodic[d] ? 1 : 0;
    L.mask.n[d] = m.N[d] * k + (L.mask.periodic[d] ? 0 : 1);
    L.h[d] = m.h[d];
  }
  for (int f = 0; f < 6; ++f) L.mask.dirichlet[f] = (m.d.bc[f] == 0 && !m.d.periodic[f / 2]) ? 1 : 0;
  L.mask.pin_first = singular ? 1 : 0;
  EXG_CHECK(L.size() < (1LL << 31), EXG_ERR_INVALID, "lattice too large");
  FE1D fe;
  fe.init(k, k + 1);
  const int n = k + 1, W = 2 * k + 1, NT = k + 2;
  L.coef.assign(3 * 2 * NT * W, 0.0);
  for (int d = 0; d < 3; ++d)
    for (int mat = 0; mat < 2; ++mat) {
      double scale = mat == 0 ? L.h[d] : 1.0 / L.h[d];
      const std::vector<double>& E = mat == 0 ? fe.M : fe.K;
      double* c = &L.coef[(d * 2 + mat) * NT * W];
      // row types 1..k-1: interior node l of one cell, columns l' - l
      for (int l = 1; l < k; ++l)
        for (int j = 0; j <= k; ++j) c[l * W + (j - l) + k] += scale * E[l * n + j];
      // type 0: vertex between two cells (local k of the left cell, local 0 of the right one)
      for (int j = 0; j <= k; ++j) {
        c[0 * W + (j - k) + k] += scale * E[k * n + j];
        c[0 * W + j + k] += scale * E[0 * n + j];
      }
      // type k: first node of a bounded line (right cell only); type k+1: last node (left cell)
      for (int j = 0; j <= k; ++j) {
        c[k * W + j + k] += scale * E[0 * n + j];
        c[(k + 1) * W + (j - k) + k] += scale * E[k * n + j];
      }
    }
}

bool lattice_constrained(const LatticeMask& m, int gx, int gy, int gz) {
  int g[3] = {gx, gy, gz};
  for (int d = 0; d < 3; ++d)
    if (!m.periodic[d] && ((g[d] == 0 && m.dirichlet[2 * d]) || (g[d] == m.n[d] - 1 && m.dirichlet[2 * d + 1])))
      return true;
  return m.pin_first && gx == 0 && gy == 0 && gz == 0;
}

__device__ __forceinline__ bool dev_constrained(const LatticeMask& m, int gx, int gy, int gz) {
  bool c = m.pin_first && gx == 0 && gy == 0 && gz == 0;
  c |= !m.periodic[0] && ((gx == 0 && m.dirichlet[0]) || (gx == m.n[0] - 1 && m.dirichlet[1]));
  c |= !m.periodic[1] && ((gy == 0 && m.dirichlet[2]) || (gy == m.n[1] - 1 && m.dirichlet[3]));
  c |= !m.periodic[2] && ((gz == 0 && m.dirichlet[4]) || (gz == m.n[2] - 1 && m.dirichlet[5]));
  return c;
}

template <int K>
__device__ __forceinline__ int row_type(int g, int n, int periodic) {
  if (!periodic) {
    if (g == 0) return K;
    if (g == n - 1) return K + 1;
  }
  return g % K;
}

// lattice coordinate of tile position g along a direction: wrapped when periodic, -1 outside
__device__ __forceinline__ int lattice_coord(int g, int n, int periodic) {
  if (periodic) return ((g % n) + n) % n;
  return (g >= 0 && g < n) ? g : -1;
}

template <int K, class T>
struct LatTile {
  static constexpr int TX = 32;
  // FP64 and high degrees: shorter register columns (no spills) and a tile that fits shared memory
  static constexpr int TY = (K <= 4 && sizeof(T) == 4) ? 8 : 4;
  static constexpr int TZ = (K <= 4 && sizeof(T) == 4) ? 8 : 4;
  static constexpr int W = 2 * K + 1, NT = K + 2;
  static constexpr int HX = TX + 2 * K, HY = TY + 2 * K, HZ = TZ + 2 * K;
  static constexpr int NCOEF = 6 * NT * W;
  static constexpr int SMEM = (NCOEF + HX * HY * HZ + 2 * HX * HY * TZ) * (int)sizeof(T);
};

template <int K, class T>
__global__ void __launch_bounds__(256) lattice_apply_kernel(const __grid_constant__ LatticeMask m,
                                                            const T* __restrict__ coef_g,
                                                            const T* __restrict__ src, T* __restrict__ dst,
                                                            const __grid_constant__ PointEpilogue ep) {
  using G = LatTile<K, T>;
  constexpr int TX = G::TX, TY = G::TY, TZ = G::TZ, W = G::W, NT = G::NT, HX = G::HX, HY = G::HY, HZ = G::HZ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* coef = reinterpret_cast<T*>(smem_raw);  // [dir][mat][type][W]
  T* in = coef + G::NCOEF;                   // HX*HY*HZ input tile; later c, d
  T* a = in + HX * HY * HZ;                  // HX*HY*TZ
  T* b = a + HX * HY * TZ;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < G::NCOEF; i += nt) coef[i] = coef_g[i];
  for (int i = tid; i < HX * HY * HZ; i += nt) {
    const int lx = i % HX, ly = (i / HX) % HY, lz = i / (HX * HY);
    const int gx = lattice_coord(x0 + lx - K, m.n[0], m.periodic[0]);
    const int gy = lattice_coord(y0 + ly - K, m.n[1], m.periodic[1]);
    const int gz = lattice_coord(z0 + lz - K, m.n[2], m.periodic[2]);
    T v = T(0);
    if (gx >= 0 && gy >= 0 && gz >= 0 && !dev_constrained(m, gx, gy, gz))
      v = src[gx + (long long)m.n[0] * (gy + (long long)m.n[1] * gz)];
    in[i] = v;
  }
  __syncthreads();
  // z pass
  {
    const T* Mz = coef + (2 * 2 + 0) * NT * W;
    const T* Kz = coef + (2 * 2 + 1) * NT * W;
    for (int col = tid; col < HX * HY; col += nt) {
      T v[HZ];
#pragma unroll
      for (int z = 0; z < HZ; ++z) v[z] = in[z * HX * HY + col];
#pragma unroll
      for (int tz = 0; tz < TZ; ++tz) {
        const int ty = row_type<K>(min(z0 + tz, m.n[2] - 1), m.n[2], m.periodic[2]);
        T sa = T(0), sb = T(0);
#pragma unroll
        for (int o = 0; o < W; ++o) {
          sa += Mz[ty * W + o] * v[tz + o];
          sb += Kz[ty * W + o] * v[tz + o];
        }
        a[tz * HX * HY + col] = sa;
        b[tz * HX * HY + col] = sb;
      }
    }
  }
  __syncthreads();
  // y pass: columns (x, z) of the haloed x range; c, d overwrite the input tile
  T* c = in;
  T* d = in + HX * TY * TZ;
  {
    const T* My = coef + (1 * 2 + 0) * NT * W;
    const T* Ky = coef + (1 * 2 + 1) * NT * W;
    for (int col = tid; col < HX * TZ; col += nt) {
      const int lx = col % HX, tz = col / HX;
      T va[HY], vb[HY];
#pragma unroll
      for (int y = 0; y < HY; ++y) {
        va[y] = a[(tz * HY + y) * HX + lx];
        vb[y] = b[(tz * HY + y) * HX + lx];
      }
#pragma unroll
      for (int ty = 0; ty < TY; ++ty) {
        const int tp = row_type<K>(min(y0 + ty, m.n[1] - 1), m.n[1], m.periodic[1]);
        T sc = T(0), sd = T(0);
#pragma unroll
        for (int o = 0; o < W; ++o) {
          sc += My[tp * W + o] * va[ty + o];
          sd += Ky[tp * W + o] * va[ty + o] + My[tp * W + o] * vb[ty + o];
        }
        c[(tz * TY + ty) * HX + lx] = sc;
        d[(tz * TY + ty) * HX + lx] = sd;
      }
    }
  }
  __syncthreads();
  // x pass and store
  const T* Mx = coef + (0 * 2 + 0) * NT * W;
  const T* Kx = coef + (0 * 2 + 1) * NT * W;
  for (int i = tid; i < TX * TY * TZ; i += nt) {
    const int tx = i % TX, ty = (i / TX) % TY, tz = i / (TX * TY);
    const int gx = x0 + tx, gy = y0 + ty, gz = z0 + tz;
    if (gx >= m.n[0] || gy >= m.n[1] || gz >= m.n[2]) continue;
    const int tp = row_type<K>(gx, m.n[0], m.periodic[0]);
    const T* cr = c + (tz * TY + ty) * HX + tx;
    const T* dr = d + (tz * TY + ty) * HX + tx;
    T s = T(0);
#pragma unroll
    for (int o = 0; o < W; ++o) s += Kx[tp * W + o] * cr[o] + Mx[tp * W + o] * dr[o];
    const long long gi = gx + (long long)m.n[0] * (gy + (long long)m.n[1] * gz);
    if (dev_constrained(m, gx, gy, gz)) s = src[gi];
    epilogue_store<T>(ep, dst, gi, src, s);
  }
}

template <int K, class T>
static void launch_apply(const LatticeHost& L, const T* src, T* dst, const PointEpilogue& ep, cudaStream_t s) {
  using G = LatTile<K, T>;
  auto kern = lattice_apply_kernel<K, T>;
  ensure_smem_attr((const void*)kern, G::SMEM);
  dim3 grid((L.mask.n[0] + G::TX - 1) / G::TX, (L.mask.n[1] + G::TY - 1) / G::TY,
            (L.mask.n[2] + G::TZ - 1) / G::TZ);
  EXG_CHECK(grid.y <= 65535 && grid.z <= 65535, EXG_ERR_UNSUPPORTED, "lattice too long in y or z");
  kern<<<grid, 256, G::SMEM, s>>>(L.mask, (const T*)L.coef_dev, src, dst, ep);
  EXG_CUDA(cudaGetLastError());
}

template <class T>
static void ensure_coef(LatticeHost& L, int prec) {
  if (L.coef_dev && L.coef_prec == prec) return;
  if (L.coef_dev) cudaFree(L.coef_dev);
  std::vector<T> c(L.coef.begin(), L.coef.end());
  EXG_CUDA(cudaMalloc(&L.coef_dev, c.size() * sizeof(T)));
  EXG_CUDA(cudaMemcpy(L.coef_dev, c.data(), c.size() * sizeof(T), cudaMemcpyHostToDevice));
  L.coef_prec = prec;
}

template <class T>
static void apply_t(LatticeHost& L, const T* src, T* dst, const PointEpilogue& ep, cudaStream_t s) {
  switch (L.k) {
#define EXG_LAT_CASE(KK) \
  case KK:               \
    launch_apply<KK, T>(L, src, dst, ep, s); \
    break;
    EXG_LAT_CASE(1)
    EXG_LAT_CASE(2)
    EXG_LAT_CASE(3)
    EXG_LAT_CASE(4)
    EXG_LAT_CASE(5)
    EXG_LAT_CASE(6)
    EXG_LAT_CASE(7)
    EXG_LAT_CASE(8)
#undef EXG_LAT_CASE
    default:
      EXG_CHECK(false, EXG_ERR_UNSUPPORTED, "continuous level degree must be 1..8");
  }
}

void lattice_prepare(LatticeHost& L, int precision) {
  if (precision == EXG_PREC_F32)
    ensure_coef<float>(L, precision);
  else
    ensure_coef<double>(L, precision);
}

void lattice_apply(LatticeHost& L, int precision, const void* src, void* dst, cudaStream_t s,
                   const PointEpilogue& ep) {
  if (precision == EXG_PREC_F32) {
    ensure_coef<float>(L, precision);
    apply_t<float>(L, (const float*)src, (float*)dst, ep, s);
  } else {
    EXG_CHECK(precision == EXG_PREC_F64, EXG_ERR_UNSUPPORTED, "continuous levels compute in FP32 or FP64");
    ensure_coef<double>(L, precision);
    apply_t<double>(L, (const double*)src, (double*)dst, ep, s);
  }
}

// ------------------------------------------------------------------------------------------
// diagonal: sum_d K_d(g_d, g_d) prod_{e != d} M_e(g_e, g_e); the band entries of a row that land
// on its own column (o = 0, and o = +-n on a periodic line of one cell); 1 on constrained nodes
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ int row_type_rt(int g, int n, int periodic, int k) {
  if (!periodic) {
    if (g == 0) return k;
    if (g == n - 1) return k + 1;
  }
  return g % k;
}

__global__ void lattice_diag_kernel(const __grid_constant__ LatticeMask m, int k, const double* __restrict__ coef,
                                    void* diag, int f32, int invert) {
  const long long total = (long long)m.n[0] * m.n[1] * m.n[2];
  const int W = 2 * k + 1, NT = k + 2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int g[3] = {(int)(i % m.n[0]), (int)((i / m.n[0]) % m.n[1]), (int)(i / ((long long)m.n[0] * m.n[1]))};
    double v = 1.0;
    if (!dev_constrained(m, g[0], g[1], g[2])) {
      double md[3], kd[3];
      for (int d = 0; d < 3; ++d) {
        const int tp = row_type_rt(g[d], m.n[d], m.periodic[d], k);
        const double* Mr = coef + ((d * 2 + 0) * NT + tp) * W;
        const double* Kr = coef + ((d * 2 + 1) * NT + tp) * W;
        md[d] = 0;
        kd[d] = 0;
        for (int o = -k; o <= k; ++o) {
          bool self = o == 0 || (m.periodic[d] && o % m.n[d] == 0);
          if (self) {
            md[d] += Mr[o + k];
            kd[d] += Kr[o + k];
          }
        }
      }
      v = kd[0] * md[1] * md[2] + md[0] * kd[1] * md[2] + md[0] * md[1] * kd[2];
      if (invert) v = fabs(v) > 1e-10 ? 1.0 / v : 1.0;
    }
    if (f32)
      static_cast<float*>(diag)[i] = (float)v;
    else
      static_cast<double*>(diag)[i] = v;
  }
}

void lattice_diagonal(LatticeHost& L, int precision, void* diag, bool invert, cudaStream_t s) {
  EXG_CHECK(precision == EXG_PREC_F32 || precision == EXG_PREC_F64, EXG_ERR_UNSUPPORTED,
            "continuous levels compute in FP32 or FP64");
  double* c = nullptr;
  EXG_CUDA(cudaMalloc(&c, L.coef.size() * sizeof(double)));
  EXG_CUDA(cudaMemcpyAsync(c, L.coef.data(), L.coef.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  const long long total = L.size();
  const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
  lattice_diag_kernel<<<std::max(blocks, 1), 256, 0, s>>>(L.mask, L.k, c, diag, precision == EXG_PREC_F32,
                                                           invert ? 1 : 0);
  EXG_CUDA(cudaGetLastError());
  EXG_CUDA(cudaStreamSynchronize(s));
  cudaFree(c);
}

// ------------------------------------------------------------------------------------------
// transfers (deal.II MGTwoLevelTransfer on FE_Q, restated: the coarse function with its
// constrained nodes read as zero is interpolated and added at the unconstrained fine nodes;
// restriction is the transpose, dropping contributions to constrained coarse nodes)
// ------------------------------------------------------------------------------------------

// one 1D pass along dir: out(.., r, ..) = sum_t val[r][t] in(.., col[r][t], ..); the first pass
// reads constrained input nodes as zero (mask_in), the last one adds into out at its
// unconstrained nodes (accumulate)
template <class T>
__global__ void lattice_pass_kernel(const T* __restrict__ in, T* __restrict__ out, int o0, int o1, int o2, int dir,
                                    int n_in_dir, const int* __restrict__ col, const T* __restrict__ val, int w,
                                    const __grid_constant__ LatticeMask min, int mask_in,
                                    const __grid_constant__ LatticeMask mout, int accumulate) {
  const long long total = (long long)o0 * o1 * o2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    int c[3] = {(int)(i % o0), (int)((i / o0) % o1), (int)(i / ((long long)o0 * o1))};
    const int r = dir == 0 ? c[0] : (dir == 1 ? c[1] : c[2]);
    int di[3] = {o0, o1, o2};
    di[dir] = n_in_dir;
    const long long stride = dir == 0 ? 1 : (dir == 1 ? (long long)di[0] : (long long)di[0] * di[1]);
    int ci[3] = {c[0], c[1], c[2]};
    ci[dir] = 0;
    const long long base = ci[0] + (long long)di[0] * (ci[1] + (long long)di[1] * ci[2]);
    T acc = T(0);
    for (int t = 0; t < w; ++t) {
      const int j = col[r * w + t];
      if (mask_in) {
        ci[dir] = j;
        if (dev_constrained(min, ci[0], ci[1], ci[2])) continue;
      }
      acc += val[r * w + t] * in[base + j * stride];
    }
    if (accumulate) {
      if (!dev_constrained(mout, c[0], c[1], c[2])) out[i] += acc;
    } else {
      out[i] = acc;
    }
  }
}

// c-transfer: every DG DoF reads its lattice node
template <class T>
__global__ void c_prolongate_kernel(const T* __restrict__ coarse, T* __restrict__ fine,
                                    const __grid_constant__ LatticeMask m, int N0, int N1, int N2, int k) {
  const int n = k + 1, n3 = n * n * n;
  const long long total = (long long)N0 * N1 * N2 * n3;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long c = i / n3;
    const int q = (int)(i % n3);
    int g[3] = {(int)(c % N0) * k + q % n, (int)((c / N0) % N1) * k + (q / n) % n,
                (int)(c / ((long long)N0 * N1)) * k + q / (n * n)};
    for (int d = 0; d < 3; ++d)
      if (m.periodic[d] && g[d] >= m.n[d]) g[d] -= m.n[d];
    if (dev_constrained(m, g[0], g[1], g[2])) continue;
    fine[i] += coarse[g[0] + (long long)m.n[0] * (g[1] + (long long)m.n[1] * g[2])];
  }
}

// c-transfer restriction: every unconstrained lattice node sums the DG DoFs at its position
// (one cell in each direction, two at a cell vertex)
template <class T>
__global__ void c_restrict_kernel(const T* __restrict__ fine, T* __restrict__ coarse,
                                  const __grid_constant__ LatticeMask m, int N0, int N1, int N2, int k) {
  const int n = k + 1;
  const int Nd[3] = {N0, N1, N2};
  const long long total = (long long)m.n[0] * m.n[1] * m.n[2];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int g[3] = {(int)(i % m.n[0]), (int)((i / m.n[0]) % m.n[1]), (int)(i / ((long long)m.n[0] * m.n[1]))};
    if (dev_constrained(m, g[0], g[1], g[2])) continue;
    int cell[3][2], loc[3][2], cnt[3];
    for (int d = 0; d < 3; ++d) {
      const int e = g[d] / k, l = g[d] % k;
      cnt[d] = 0;
      if (l != 0) {
        cell[d][0] = e;
        loc[d][0] = l;
        cnt[d] = 1;
        continue;
      }
      if (e >= 1 || m.periodic[d]) {  // left cell, its last node
        cell[d][cnt[d]] = e >= 1 ? e - 1 : Nd[d] - 1;
        loc[d][cnt[d]] = k;
        ++cnt[d];
      }
      if (e < Nd[d]) {  // right cell, its first node
        cell[d][cnt[d]] = e;
        loc[d][cnt[d]] = 0;
        ++cnt[d];
      }
    }
    T acc = T(0);
    for (int cz = 0; cz < cnt[2]; ++cz)
      for (int cy = 0; cy < cnt[1]; ++cy)
        for (int cx = 0; cx < cnt[0]; ++cx) {
          const long long c = cell[0][cx] + (long long)N0 * (cell[1][cy] + (long long)N1 * cell[2][cz]);
          acc += fine[c * n * n * n + loc[0][cx] + n * (loc[1][cy] + n * loc[2][cz])];
        }
    coarse[i] += acc;
  }
}

static int grid_for(long long total) {
  return (int)std::max<long long>(1, std::min<long long>((total + 255) / 256, 152LL * 32));
}

LatticeTransfer::~LatticeTransfer() {
  for (int d = 0; d < 3; ++d)
    for (void* p : {(void*)pcol[d], (void*)rcol[d], pval[d], rval[d]})
      if (p) cudaFree(p);
  for (void* p : scratch)
    if (p) cudaFree(p);
}

template <class T>
static void upload_table(const std::vector<int>& cols, const std::vector<double>& vals, int** dc, void** dv) {
  std::vector<T> v(vals.begin(), vals.end());
  EXG_CUDA(cudaMalloc(dc, cols.size() * sizeof(int)));
  EXG_CUDA(cudaMalloc(dv, v.size() * sizeof(T)));
  EXG_CUDA(cudaMemcpy(*dc, cols.data(), cols.size() * sizeof(int), cudaMemcpyHostToDevice));
  EXG_CUDA(cudaMemcpy(*dv, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
}

void LatticeTransfer::setup(const LatticeHost& coarse, const LatticeHost& fine, int precision) {
  EXG_CHECK(precision == EXG_PREC_F32 || precision == EXG_PREC_F64, EXG_ERR_UNSUPPORTED,
            "continuous levels compute in FP32 or FP64");
  prec = precision;
  mc = coarse.mask;
  mf = fine.mask;
  kc = coarse.k;
  kf = fine.k;
  const std::vector<double> zc = gauss_lobatto(kc + 1), zf = gauss_lobatto(kf + 1);
  for (int d = 0; d < 3; ++d) {
    const int Ncd = coarse.N[d], Nfd = fine.N[d], nf = mf.n[d], nc = mc.n[d];
    const bool per = mc.periodic[d] != 0, is_h = Nfd != Ncd;
    EXG_CHECK(Nfd == Ncd || Nfd == 2 * Ncd, EXG_ERR_UNSUPPORTED, "unsupported continuous transfer");
    // prolongation rows: fine node -> kc+1 coarse nodes of the coarse cell around it
    const int w = kc + 1;
    std::vector<int> pc((size_t)nf * w, 0);
    std::vector<double> pv((size_t)nf * w, 0.0);
    std::vector<char> done(nf, 0);
    for (int ef = 0; ef < Nfd; ++ef)
      for (int i = 0; i <= kf; ++i) {
        int g = ef * kf + i;
        if (per) g %= nf;
        if (done[g]) continue;
        done[g] = 1;
        const int ec = is_h ? ef / 2 : ef;
        const double xi = is_h ? 0.5 * ((ef % 2) + zf[i]) : zf[i];
        for (int j = 0; j <= kc; ++j) {
          int cg = ec * kc + j;
          if (per) cg %= nc;
          pc[(size_t)g * w + j] = cg;
          pv[(size_t)g * w + j] = lagrange(zc, j, xi);
        }
      }
    // restriction rows: the transpose, padded to the widest coarse row
    std::vector<std::vector<std::pair<int, double>>> rows(nc);
    for (int g = 0; g < nf; ++g)
      for (int j = 0; j < w; ++j) rows[pc[(size_t)g * w + j]].push_back({g, pv[(size_t)g * w + j]});
    int wr_d = 1;
    for (auto& r : rows) wr_d = std::max(wr_d, (int)r.size());
    std::vector<int> rc((size_t)nc * wr_d, 0);
    std::vector<double> rv((size_t)nc * wr_d, 0.0);
    for (int j = 0; j < nc; ++j)
      for (size_t t = 0; t < rows[j].size(); ++t) {
        rc[(size_t)j * wr_d + t] = rows[j][t].first;
        rv[(size_t)j * wr_d + t] = rows[j][t].second;
      }
    wp[d] = w;
    wr[d] = wr_d;
    if (prec == EXG_PREC_F32) {
      upload_table<float>(pc, pv, &pcol[d], &pval[d]);
      upload_table<float>(rc, rv, &rcol[d], &rval[d]);
    } else {
      upload_table<double>(pc, pv, &pcol[d], &pval[d]);
      upload_table<double>(rc, rv, &rcol[d], &rval[d]);
    }
  }
  const size_t words = (size_t)mf.n[0] * mf.n[1] * mc.n[2];
  const size_t bytes = words * (prec == EXG_PREC_F32 ? 4 : 8);
  EXG_CUDA(cudaMalloc(&scratch[0], bytes));
  EXG_CUDA(cudaMalloc(&scratch[1], bytes));
}

void LatticeTransfer::setup_dg(const LatticeHost& coarse, int precision) {
  EXG_CHECK(precision == EXG_PREC_F32 || precision == EXG_PREC_F64, EXG_ERR_UNSUPPORTED,
            "continuous levels compute in FP32 or FP64");
  to_dg = true;
  prec = precision;
  mc = coarse.mask;
  kc = kf = coarse.k;
  for (int d = 0; d < 3; ++d) Nc[d] = coarse.N[d];
}

template <class T>
static void pass(const LatticeTransfer& t, const T* in, T* out, const int dims_out[3], int dir, int n_in_dir,
                 const int* col, const void* val, int w, const LatticeMask* min, const LatticeMask* mout,
                 cudaStream_t s) {
  const long long total = (long long)dims_out[0] * dims_out[1] * dims_out[2];
  LatticeMask none{};
  lattice_pass_kernel<T><<<grid_for(total), 256, 0, s>>>(in, out, dims_out[0], dims_out[1], dims_out[2], dir, n_in_dir,
                                                         col, (const T*)val, w, min ? *min : none, min ? 1 : 0,
                                                         mout ? *mout : none, mout ? 1 : 0);
  EXG_CUDA(cudaGetLastError());
  (void)t;
}

template <class T>
static void prolongate_t(const LatticeTransfer& t, const T* coarse, T* fine, cudaStream_t s) {
  if (t.to_dg) {
    const long long total = (long long)t.Nc[0] * t.Nc[1] * t.Nc[2] * (t.kc + 1) * (t.kc + 1) * (t.kc + 1);
    c_prolongate_kernel<T><<<grid_for(total), 256, 0, s>>>(coarse, fine, t.mc, t.Nc[0], t.Nc[1], t.Nc[2], t.kc);
    EXG_CUDA(cudaGetLastError());
    return;
  }
  T* s0 = (T*)t.scratch[0];
  T* s1 = (T*)t.scratch[1];
  const int d0[3] = {t.mf.n[0], t.mc.n[1], t.mc.n[2]};
  const int d1[3] = {t.mf.n[0], t.mf.n[1], t.mc.n[2]};
  const int d2[3] = {t.mf.n[0], t.mf.n[1], t.mf.n[2]};
  pass<T>(t, coarse, s0, d0, 0, t.mc.n[0], t.pcol[0], t.pval[0], t.wp[0], &t.mc, nullptr, s);
  pass<T>(t, s0, s1, d1, 1, t.mc.n[1], t.pcol[1], t.pval[1], t.wp[1], nullptr, nullptr, s);
  pass<T>(t, s1, fine, d2, 2, t.mc.n[2], t.pcol[2], t.pval[2], t.wp[2], nullptr, &t.mf, s);
}

template <class T>
static void restrict_t(const LatticeTransfer& t, const T* fine, T* coarse, cudaStream_t s) {
  if (t.to_dg) {
    c_restrict_kernel<T><<<grid_for((long long)t.mc.n[0] * t.mc.n[1] * t.mc.n[2]), 256, 0, s>>>(
        fine, coarse, t.mc, t.Nc[0], t.Nc[1], t.Nc[2], t.kc);
    EXG_CUDA(cudaGetLastError());
    return;
  }
  T* s0 = (T*)t.scratch[0];
  T* s1 = (T*)t.scratch[1];
  const int d0[3] = {t.mf.n[0], t.mf.n[1], t.mc.n[2]};
  const int d1[3] = {t.mf.n[0], t.mc.n[1], t.mc.n[2]};
  const int d2[3] = {t.mc.n[0], t.mc.n[1], t.mc.n[2]};
  pass<T>(t, fine, s0, d0, 2, t.mf.n[2], t.rcol[2], t.rval[2], t.wr[2], &t.mf, nullptr, s);
  pass<T>(t, s0, s1, d1, 1, t.mf.n[1], t.rcol[1], t.rval[1], t.wr[1], nullptr, nullptr, s);
  pass<T>(t, s1, coarse, d2, 0, t.mf.n[0], t.rcol[0], t.rval[0], t.wr[0], nullptr, &t.mc, s);
}

void LatticeTransfer::prolongate_add(const void* coarse, void* fine, cudaStream_t s) const {
  if (prec == EXG_PREC_F32)
    prolongate_t<float>(*this, (const float*)coarse, (float*)fine, s);
  else
    prolongate_t<double>(*this, (const double*)coarse, (double*)fine, s);
}

void LatticeTransfer::restrict_add(const void* fine, void* coarse, cudaStream_t s) const {
  if (prec == EXG_PREC_F32)
    restrict_t<float>(*this, (const float*)fine, (float*)coarse, s);
  else
    restrict_t<double>(*this, (const double*)fine, (double*)coarse, s);
}

}  // namespace exg
