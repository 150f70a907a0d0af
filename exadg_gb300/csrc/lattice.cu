// Continuous levels of cphMG on Cartesian meshes (declarations and the algorithm in lattice.h).
//
// Apply: one CTA per TX x TY x TZ tile of output nodes (extents and origins multiples of k, so
// every row type is a compile-time constant and the unit-cell band coefficients are FMA operands
// from the constant bank).  The tile and a halo of k nodes per side are read once into shared
// memory (a warp per row, several rows in flight; nodes outside a bounded lattice read as zero,
// periodic directions wrapped, constrained nodes zeroed afterwards), then three 1D band passes:
//   z: a = M_z x, b = K_z x            (a thread per (x, y) column, the column in registers;
//                                       a, b written over the tile where they fit)
//   y: c = M_y a, d = K_y a + M_y b    (a thread per (x, z) column)
//   x: A x = K_x c + M_x d             (a thread per row segment of k nodes)
// and a coalesced store through the point epilogue (constrained nodes store src).
// Global traffic is one read of src (plus the halo, mostly from L2) and one write of dst.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <set>
#include <type_traits>

#include "epilogue.cuh"
#include "lattice.h"

namespace exg {

void make_lattice(const MeshInfo& m, int k, bool singular, LatticeHost& L) {
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

// lattice coordinate of tile position g along a direction: wrapped when periodic, -1 outside
__device__ __forceinline__ int lattice_coord(int g, int n, int periodic) {
  if (periodic) return ((g % n) + n) % n;
  return (g >= 0 && g < n) ? g : -1;
}

// Band tables of the unit cell for every degree, in constant memory: for degree K,
// [mat (0 mass, 1 stiffness)][row type t = g mod K][o + K], o = -K..K, then the diagonal
// corrections of a bounded line's first and last node [mat][2].  With tiles whose origin and
// extent are multiples of K, every row type in the unrolled passes is a compile-time constant,
// so each coefficient is an FMA operand from the constant bank.
__host__ __device__ constexpr int band_size(int K) { return 2 * K * (2 * K + 1) + 4; }
__host__ __device__ constexpr int band_off(int K) {
  int s = 0;
  for (int k = 1; k < K; ++k) s += band_size(k);
  return s;
}
constexpr int BAND_TOTAL = band_off(LAT_KMAX + 1);
__constant__ float c_band_f[BAND_TOTAL];
__constant__ double c_band_d[BAND_TOTAL];

template <class T>
__device__ __forceinline__ T band(int i);
template <>
__device__ __forceinline__ float band<float>(int i) {
  return c_band_f[i];
}
template <>
__device__ __forceinline__ double band<double>(int i) {
  return c_band_d[i];
}

// unit-cell band table of degree K (row types 0..K-1; a bounded line's end nodes are type 0 rows
// whose outside neighbours are zero, minus the other cell's diagonal entry)
static void unit_band(int K, std::vector<double>& out) {
  FE1D fe;
  fe.init(K, K + 1);
  const int n = K + 1, W = 2 * K + 1;
  out.assign(band_size(K), 0.0);
  for (int mat = 0; mat < 2; ++mat) {
    const std::vector<double>& E = mat == 0 ? fe.M : fe.K;
    double* c = &out[mat * K * W];
    for (int t = 1; t < K; ++t)
      for (int j = 0; j <= K; ++j) c[t * W + (j - t) + K] += E[t * n + j];
    for (int j = 0; j <= K; ++j) {
      c[(j - K) + K] += E[K * n + j];
      c[j + K] += E[0 * n + j];
    }
    out[2 * K * W + mat * 2 + 0] = E[K * n + K];  // first node: no left cell
    out[2 * K * W + mat * 2 + 1] = E[0 * n + 0];  // last node: no right cell
  }
}

void lattice_prepare(LatticeHost& L, int precision) {
  (void)L;
  (void)precision;
  static std::mutex mu;
  static std::set<int> done;
  int dev = 0;
  EXG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if (done.count(dev)) return;
  std::vector<double> all(BAND_TOTAL, 0.0), one;
  for (int K = 1; K <= LAT_KMAX; ++K) {
    unit_band(K, one);
    std::copy(one.begin(), one.end(), all.begin() + band_off(K));
  }
  std::vector<float> allf(all.begin(), all.end());
  EXG_CUDA(cudaMemcpyToSymbol(c_band_d, all.data(), all.size() * sizeof(double)));
  EXG_CUDA(cudaMemcpyToSymbol(c_band_f, allf.data(), allf.size() * sizeof(float)));
  done.insert(dev);
}

template <class T>
struct LatParams {
  LatticeMask m;
  T hm[3], hk[3];  // mass scale h_d and stiffness scale 1 / h_d
};

// the largest multiple of K not above `want` (at least K)
__host__ __device__ constexpr int tile_mult(int K, int want) { return K * (want / K > 0 ? want / K : 1); }

// SMALL: quarter-size tiles for lattices too small to fill the GPU with full ones
template <int K, class T, bool SMALL>
struct LatTile {
  static constexpr bool F32 = sizeof(T) == 4 && !SMALL;
  static constexpr int TX = F32 ? tile_mult(K, 32) : (K <= 4 ? tile_mult(K, 16) : tile_mult(K, 8));
  static constexpr int TY = F32 ? tile_mult(K, 8) : tile_mult(K, 4);
  static constexpr int TZ = TY;
  static constexpr int W = 2 * K + 1;
  static constexpr int HX = TX + 2 * K, HY = TY + 2 * K, HZ = TZ + 2 * K;
  static constexpr int HXP = HX | 1;  // odd row stride of c, d (conflict-free x pass)
  static constexpr int TXP = TX | 1;  // odd row stride of the x pass results
  // Shared-memory layout.  INPLACE (TZ <= 2K): the z pass writes a and b over the input tile (a
  // thread owns its column: all of it is in registers before the writes), c and d follow the
  // tile, the x pass results go back into the tile.  Otherwise a and b follow the tile and c, d
  // and the results reuse the tile and a.
  static constexpr bool INPLACE = 2 * TZ <= HZ;
  static constexpr int TILE = HX * HY * HZ, PLANE = HX * HY, CD = HXP * TY * TZ;
  static constexpr int IN_WORDS = INPLACE ? TILE : (TILE > 2 * CD ? TILE : 2 * CD);
  static constexpr int A_OFF = INPLACE ? 0 : IN_WORDS;
  static constexpr int B_OFF = A_OFF + PLANE * TZ;
  static constexpr int C_OFF = INPLACE ? TILE : 0;
  static constexpr int D_OFF = C_OFF + CD;
  static constexpr int RES_OFF = INPLACE ? 0 : A_OFF;
  static constexpr int SMEM = (INPLACE ? TILE + 2 * CD : IN_WORDS + 2 * PLANE * TZ) * (int)sizeof(T);
  static_assert(TXP * TY * TZ <= HX * HY * TZ, "results must fit a");
  static_assert(!INPLACE || 2 * PLANE * TZ <= TILE, "a, b must fit the tile");
};

// compile-time loop: f(std::integral_constant<int, I>) for I = B..E-1
template <int B, int E, class F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

// row g of a 1D band pass on the column v (v[T0 + o + K] = x_{g+o}), row type T0 mod K: mass and
// stiffness sums of the unit cell (every coefficient index a constant, so the coefficient is an
// FMA operand from the constant bank), with the diagonal correction of a bounded line's end nodes
template <int K, int T0, bool WANT_K, class T>
__device__ __forceinline__ void band_row(const T* v, int g, int n, int periodic, T& sm, T& sk) {
  constexpr int W = 2 * K + 1, B = band_off(K), t = T0 % K;
  sm = T(0);
  sk = T(0);
  static_for<0, W>([&](auto oc) {
    constexpr int o = decltype(oc)::value;
    if constexpr (t == 0 || (o >= K - t && o <= 2 * K - t)) {
      sm += band<T>(B + (0 * K + t) * W + o) * v[T0 + o];
      if constexpr (WANT_K) sk += band<T>(B + (1 * K + t) * W + o) * v[T0 + o];
    }
  });
  if constexpr (t == 0) {
    if (!periodic && (g == 0 || g == n - 1)) {
      const bool first = g == 0;
      sm -= (first ? band<T>(B + 2 * K * W + 0) : band<T>(B + 2 * K * W + 1)) * v[T0 + K];
      if constexpr (WANT_K) sk -= (first ? band<T>(B + 2 * K * W + 2) : band<T>(B + 2 * K * W + 3)) * v[T0 + K];
    }
  }
}

template <int K, class T, bool SMALL>
__global__ void __launch_bounds__(256) lattice_apply_kernel(const __grid_constant__ LatParams<T> P,
                                                            const T* __restrict__ src, T* __restrict__ dst,
                                                            const __grid_constant__ PointEpilogue ep) {
  using G = LatTile<K, T, SMALL>;
  constexpr int TX = G::TX, TY = G::TY, TZ = G::TZ, HX = G::HX, HY = G::HY, HZ = G::HZ, HXP = G::HXP,
                TXP = G::TXP, NTH = 256;
  const LatticeMask& m = P.m;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* in = reinterpret_cast<T*>(smem_raw);  // HX*HY*HZ input tile
  T* a = in + G::A_OFF;                    // HX*HY*TZ z pass results
  T* b = in + G::B_OFF;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
  const int tid = threadIdx.x;
  // tile load: a warp per row of HX nodes, U rows in flight per warp; a lane's (at most two) x
  // positions are found once.  Constrained nodes are zeroed afterwards, in the tiles that hold any.
  const int lane = tid & 31, warp = tid >> 5;
  static_assert(HX <= 64, "two x positions per lane");
  constexpr int U = sizeof(T) == 4 ? 8 : 4, ROWS_IN = HY * HZ;
  // tiles whose haloed box lies inside the lattice (most of them) need no wrap or range test
  const bool interior = x0 >= K && x0 - K + HX <= m.n[0] && y0 >= K && y0 - K + HY <= m.n[1] && z0 >= K &&
                        z0 - K + HZ <= m.n[2];
  if (interior) {
    const T* base = src + ((x0 - K) + m.n[0] * ((y0 - K) + m.n[1] * (z0 - K)));
    for (int r0 = warp * U; r0 < ROWS_IN; r0 += (NTH / 32) * U) {
      T vals[U][2];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int r = r0 + u;
        const T* rp = base + m.n[0] * (r % HY + m.n[1] * (r / HY));
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int lx = lane + 32 * c;
          vals[u][c] = (r < ROWS_IN && lx < HX) ? rp[lx] : T(0);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int lx = lane + 32 * c;
          if (r0 + u < ROWS_IN && lx < HX) in[(r0 + u) * HX + lx] = vals[u][c];
        }
    }
  }
  int gxs[2];
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const int lx = lane + 32 * c;
    gxs[c] = lx < HX ? lattice_coord(x0 + lx - K, m.n[0], m.periodic[0]) : -1;
  }
  if (!interior)
  for (int r0 = warp * U; r0 < ROWS_IN; r0 += (NTH / 32) * U) {
    T vals[U][2];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int r = r0 + u;
      const int ly = r % HY, lz = r / HY;
      const int gy = lattice_coord(y0 + ly - K, m.n[1], m.periodic[1]);
      const int gz = lattice_coord(z0 + lz - K, m.n[2], m.periodic[2]);
      const bool rok = r < ROWS_IN && gy >= 0 && gz >= 0;
      const int rbase = m.n[0] * (gy + m.n[1] * gz);
#pragma unroll
      for (int c = 0; c < 2; ++c) vals[u][c] = (rok && gxs[c] >= 0) ? src[rbase + gxs[c]] : T(0);
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int lx = lane + 32 * c;
        if (r0 + u < ROWS_IN && lx < HX) in[(r0 + u) * HX + lx] = vals[u][c];
      }
  }
  __syncthreads();
  {
    // Dirichlet planes inside the tile (tile position of lattice plane 0 and n-1 per direction)
    int plane[6];
    bool any = false;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const int dir = f / 2, o0 = dir == 0 ? x0 : (dir == 1 ? y0 : z0), H = dir == 0 ? HX : (dir == 1 ? HY : HZ);
      const int lp = (f % 2 == 0 ? 0 : m.n[dir] - 1) - o0 + K;
      plane[f] = (!m.periodic[dir] && m.dirichlet[f] && lp >= 0 && lp < H) ? lp : -1;
      any |= plane[f] >= 0;
    }
    if (any) {
#pragma unroll
      for (int f = 0; f < 6; ++f) {
        if (plane[f] < 0) continue;
        const int dir = f / 2;
        const int na = dir == 0 ? HY : HX, nb = dir == 2 ? HY : HZ;  // the plane's other two extents
        for (int i = tid; i < na * nb; i += NTH) {
          const int ia = i % na, ib = i / na;
          const int lx = dir == 0 ? plane[f] : ia, ly = dir == 1 ? plane[f] : (dir == 0 ? ia : ib),
                    lz = dir == 2 ? plane[f] : ib;
          in[(lz * HY + ly) * HX + lx] = T(0);
        }
      }
    }
    // node 0 of a singular operator (wherever periodic copies of it sit in the tile)
    bool pin = m.pin_first;
#pragma unroll
    for (int dir = 0; dir < 3; ++dir) {
      const int o = (dir == 0 ? x0 : (dir == 1 ? y0 : z0)) - K, H = dir == 0 ? HX : (dir == 1 ? HY : HZ);
      const int first = m.periodic[dir] ? ((-o) % m.n[dir] + m.n[dir]) % m.n[dir] : -o;  // tile position of 0
      pin = pin && first >= 0 && first < H;
    }
    if (pin && tid == 0) {
      for (int lz = 0; lz < HZ; ++lz)
        if (lattice_coord(z0 + lz - K, m.n[2], m.periodic[2]) == 0)
          for (int ly = 0; ly < HY; ++ly)
            if (lattice_coord(y0 + ly - K, m.n[1], m.periodic[1]) == 0)
              for (int lx = 0; lx < HX; ++lx)
                if (lattice_coord(x0 + lx - K, m.n[0], m.periodic[0]) == 0) in[(lz * HY + ly) * HX + lx] = T(0);
    }
    if (any || pin) __syncthreads();
  }
  // z pass: a = M_z x, b = K_z x on the haloed (x, y) plane
  for (int col = tid; col < HX * HY; col += NTH) {
    T v[HZ];
#pragma unroll
    for (int z = 0; z < HZ; ++z) v[z] = in[z * HX * HY + col];
    static_for<0, TZ>([&](auto tc) {
      constexpr int tz = decltype(tc)::value;
      T sm, sk;
      band_row<K, tz, true, T>(v, z0 + tz, m.n[2], m.periodic[2], sm, sk);
      a[tz * HX * HY + col] = sm * P.hm[2];
      b[tz * HX * HY + col] = sk * P.hk[2];
    });
  }
  __syncthreads();
  // y pass: c = M_y a, d = K_y a + M_y b on the haloed x range
  T* c = in + G::C_OFF;
  T* d = in + G::D_OFF;
  for (int col = tid; col < HX * TZ; col += NTH) {
    const int lx = col % HX, tz = col / HX;
    T va[HY], vb[HY];
#pragma unroll
    for (int y = 0; y < HY; ++y) {
      va[y] = a[(tz * HY + y) * HX + lx];
      vb[y] = b[(tz * HY + y) * HX + lx];
    }
    static_for<0, TY>([&](auto tc) {
      constexpr int ty = decltype(tc)::value;
      T ma, ka, mb, kb;
      band_row<K, ty, true, T>(va, y0 + ty, m.n[1], m.periodic[1], ma, ka);
      band_row<K, ty, false, T>(vb, y0 + ty, m.n[1], m.periodic[1], mb, kb);
      c[(tz * TY + ty) * HXP + lx] = ma * P.hm[1];
      d[(tz * TY + ty) * HXP + lx] = ka * P.hk[1] + mb * P.hm[1];
    });
  }
  __syncthreads();
  // x pass: a thread per (row, cell segment of K nodes), rows across the lanes
  T* res = in + G::RES_OFF;
  constexpr int SEG = TX / K, ROWS = TY * TZ;
  for (int it = tid; it < SEG * ROWS; it += NTH) {
    const int row = it % ROWS, q = it / ROWS;
    const T* cr = c + row * HXP + q * K;
    const T* dr = d + row * HXP + q * K;
    T vc[3 * K], vd[3 * K];
#pragma unroll
    for (int j = 0; j < 3 * K; ++j) {
      vc[j] = cr[j];
      vd[j] = dr[j];
    }
    const int gq = x0 + q * K;
    static_for<0, K>([&](auto lc) {
      constexpr int l = decltype(lc)::value;
      T mc, kc, md, kd;
      band_row<K, l, true, T>(vc, gq + l, m.n[0], m.periodic[0], mc, kc);
      band_row<K, l, false, T>(vd, gq + l, m.n[0], m.periodic[0], md, kd);
      res[row * TXP + q * K + l] = kc * P.hk[0] + md * P.hm[0];
    });
  }
  __syncthreads();
  // coalesced store through the point epilogue, a warp per output row (U rows in flight);
  // constrained nodes keep src
  static_assert(TX <= 32, "one x position per lane");
  const int gx = x0 + lane;
  const bool xin = lane < TX && gx < m.n[0];
  const bool xc = !m.periodic[0] && ((gx == 0 && m.dirichlet[0]) || (gx == m.n[0] - 1 && m.dirichlet[1]));
  constexpr int ROWS_OUT = TY * TZ;
  for (int r0 = warp * U; r0 < ROWS_OUT; r0 += (NTH / 32) * U) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int row = r0 + u;
      const int ty = row % TY, tz = row / TY;
      const int gy = y0 + ty, gz = z0 + tz;
      if (row >= ROWS_OUT || !xin || gy >= m.n[1] || gz >= m.n[2]) continue;
      const bool rc = (!m.periodic[1] && ((gy == 0 && m.dirichlet[2]) || (gy == m.n[1] - 1 && m.dirichlet[3]))) ||
                      (!m.periodic[2] && ((gz == 0 && m.dirichlet[4]) || (gz == m.n[2] - 1 && m.dirichlet[5])));
      const int gi = gx + m.n[0] * (gy + m.n[1] * gz);
      T v = res[row * TXP + lane];
      if (xc || rc || (m.pin_first && gx == 0 && gy == 0 && gz == 0)) v = src[gi];
      epilogue_store<T>(ep, dst, gi, src, v);
    }
  }
}

template <int K, class T, bool SMALL>
static void launch_apply(const LatticeHost& L, const T* src, T* dst, const PointEpilogue& ep, cudaStream_t s) {
  using G = LatTile<K, T, SMALL>;
  auto kern = lattice_apply_kernel<K, T, SMALL>;
  ensure_smem_attr((const void*)kern, G::SMEM);
  dim3 grid((L.mask.n[0] + G::TX - 1) / G::TX, (L.mask.n[1] + G::TY - 1) / G::TY,
            (L.mask.n[2] + G::TZ - 1) / G::TZ);
  EXG_CHECK(grid.y <= 65535 && grid.z <= 65535, EXG_ERR_UNSUPPORTED, "lattice too long in y or z");
  LatParams<T> P;
  P.m = L.mask;
  for (int e = 0; e < 3; ++e) {
    P.hm[e] = (T)L.h[e];
    P.hk[e] = (T)(1.0 / L.h[e]);
  }
  kern<<<grid, 256, G::SMEM, s>>>(P, src, dst, ep);
  EXG_CUDA(cudaGetLastError());
}

// full-size tiles of a lattice
template <int K, class T>
static long long tiles(const LatticeHost& L) {
  using G = LatTile<K, T, false>;
  return (long long)((L.mask.n[0] + G::TX - 1) / G::TX) * ((L.mask.n[1] + G::TY - 1) / G::TY) *
         ((L.mask.n[2] + G::TZ - 1) / G::TZ);
}

template <class T>
static void apply_t(LatticeHost& L, const T* src, T* dst, const PointEpilogue& ep, cudaStream_t s) {
  switch (L.k) {
#define EXG_LAT_CASE(KK)                                                    \
  case KK:                                                                  \
    if (tiles<KK, T>(L) < 152)                                              \
      launch_apply<KK, T, true>(L, src, dst, ep, s);                        \
    else                                                                    \
      launch_apply<KK, T, false>(L, src, dst, ep, s);                       \
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

// Q1 lattices (every h-level of cphMG): a thread per node evaluates the (2K+1)^3-point stencil
// from global memory (neighbours are L1/L2 hits) in one launch without the tile pipeline's
// barriers, which make the tile kernel latency-bound on the small coarse lattices
__device__ __forceinline__ int wrap_or_out(int g, int n, int periodic) {
  if (g >= 0 && g < n) return g;
  if (!periodic) return -1;
  return ((g % n) + n) % n;
}

template <int K, class T>
__global__ void __launch_bounds__(256) lattice_direct_kernel(const __grid_constant__ LatParams<T> P,
                                                             const T* __restrict__ src, T* __restrict__ dst,
                                                             const __grid_constant__ PointEpilogue ep) {
  constexpr int W = 2 * K + 1, B = band_off(K);
  const LatticeMask& m = P.m;
  const int total = m.n[0] * m.n[1] * m.n[2];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int g[3] = {i % m.n[0], (i / m.n[0]) % m.n[1], i / (m.n[0] * m.n[1])};
    // per direction: neighbour coordinates (-1 outside), their Dirichlet flags, the mass and
    // stiffness rows of the node's row type (vertex rows at a bounded line's end without the
    // missing cell's diagonal entry)
    int nb[3][W];
    bool fc[3][W];
    T mm[3][W], kk[3][W];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int n = m.n[d], per = m.periodic[d], t = g[d] % K;
#pragma unroll
      for (int o = 0; o < W; ++o) {
        const int c = wrap_or_out(g[d] + o - K, n, per);
        nb[d][o] = c;
        fc[d][o] = !per && ((c == 0 && m.dirichlet[2 * d]) || (c == n - 1 && m.dirichlet[2 * d + 1]));
        mm[d][o] = band<T>(B + (0 * K + t) * W + o) * P.hm[d];
        kk[d][o] = band<T>(B + (1 * K + t) * W + o) * P.hk[d];
      }
      if (!per && g[d] == 0) {
        mm[d][K] -= band<T>(B + 2 * K * W + 0) * P.hm[d];
        kk[d][K] -= band<T>(B + 2 * K * W + 2) * P.hk[d];
      }
      if (!per && g[d] == n - 1) {
        mm[d][K] -= band<T>(B + 2 * K * W + 1) * P.hm[d];
        kk[d][K] -= band<T>(B + 2 * K * W + 3) * P.hk[d];
      }
    }
    T acc = T(0);
#pragma unroll
    for (int c = 0; c < W; ++c)
#pragma unroll
      for (int b = 0; b < W; ++b) {
        T sx = T(0), tx = T(0);  // sum_a K_x x, sum_a M_x x along the row (b, c)
        const bool rowok = nb[1][b] >= 0 && nb[2][c] >= 0 && !fc[1][b] && !fc[2][c];
        const int rbase = m.n[0] * (nb[1][b] + m.n[1] * nb[2][c]);
#pragma unroll
        for (int a = 0; a < W; ++a) {
          const bool ok = rowok && nb[0][a] >= 0 && !fc[0][a] &&
                          !(m.pin_first && nb[0][a] == 0 && nb[1][b] == 0 && nb[2][c] == 0);
          const T x = ok ? src[rbase + nb[0][a]] : T(0);
          sx += kk[0][a] * x;
          tx += mm[0][a] * x;
        }
        acc += sx * mm[1][b] * mm[2][c] + tx * (kk[1][b] * mm[2][c] + mm[1][b] * kk[2][c]);
      }
    const bool con = (!m.periodic[0] && ((g[0] == 0 && m.dirichlet[0]) || (g[0] == m.n[0] - 1 && m.dirichlet[1]))) ||
                     (!m.periodic[1] && ((g[1] == 0 && m.dirichlet[2]) || (g[1] == m.n[1] - 1 && m.dirichlet[3]))) ||
                     (!m.periodic[2] && ((g[2] == 0 && m.dirichlet[4]) || (g[2] == m.n[2] - 1 && m.dirichlet[5]))) ||
                     (m.pin_first && i == 0);
    if (con) acc = src[i];
    epilogue_store<T>(ep, dst, i, src, acc);
  }
}

template <int K, class T>
static void apply_direct(const LatticeHost& L, const T* src, T* dst, const PointEpilogue& ep, cudaStream_t s) {
  LatParams<T> P;
  P.m = L.mask;
  for (int e = 0; e < 3; ++e) {
    P.hm[e] = (T)L.h[e];
    P.hk[e] = (T)(1.0 / L.h[e]);
  }
  const long long total = L.size();
  const int blocks = (int)std::max<long long>(1, std::min<long long>((total + 255) / 256, 152LL * 16));
  lattice_direct_kernel<K, T><<<blocks, 256, 0, s>>>(P, src, dst, ep);
  EXG_CUDA(cudaGetLastError());
}

// the direct kernel for Q1 (measured: at Q2 its 125 loads per node make it slower than the tiles)
static bool use_direct(const LatticeHost& L) { return L.k == 1; }

void lattice_apply(LatticeHost& L, int precision, const void* src, void* dst, cudaStream_t s,
                   const PointEpilogue& ep) {
  if (precision == EXG_PREC_F32) {
    if (use_direct(L))
      L.k == 1 ? apply_direct<1, float>(L, (const float*)src, (float*)dst, ep, s)
               : apply_direct<2, float>(L, (const float*)src, (float*)dst, ep, s);
    else
      apply_t<float>(L, (const float*)src, (float*)dst, ep, s);
  } else {
    EXG_CHECK(precision == EXG_PREC_F64, EXG_ERR_UNSUPPORTED, "continuous levels compute in FP32 or FP64");
    if (use_direct(L))
      L.k == 1 ? apply_direct<1, double>(L, (const double*)src, (double*)dst, ep, s)
               : apply_direct<2, double>(L, (const double*)src, (double*)dst, ep, s);
    else
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

// one 1D pass along dir: out(.., r, ..) = sum_t val[r][t] in(.., col[r][t], ..) with W taps per
// row (rows padded with zero taps; W a compile-time constant so that all loads of a row are in
// flight together); the first pass reads constrained input nodes as zero (mask_in), the last one
// adds into out at its unconstrained nodes (accumulate).  Extents are below 2^31.
template <class T, int W>
__global__ void lattice_pass_kernel(const T* __restrict__ in, T* __restrict__ out, int o0, int o1, int o2, int dir,
                                    int n_in_dir, const int* __restrict__ col, const T* __restrict__ val,
                                    const __grid_constant__ LatticeMask min, int mask_in,
                                    const __grid_constant__ LatticeMask mout, int accumulate) {
  const int total = o0 * o1 * o2;
  const int i0 = dir == 0 ? n_in_dir : o0;  // input extents
  const int i1 = dir == 1 ? n_in_dir : o1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int cx = i % o0, rest = i / o0, cy = rest % o1, cz = rest / o1;
    const int r = dir == 0 ? cx : (dir == 1 ? cy : cz);
    const int stride = dir == 0 ? 1 : (dir == 1 ? i0 : i0 * i1);
    const int base = (dir == 0 ? 0 : cx) + i0 * ((dir == 1 ? 0 : cy) + i1 * (dir == 2 ? 0 : cz));
    int cs[W];
    T vs[W], xs[W];
#pragma unroll
    for (int t = 0; t < W; ++t) {
      cs[t] = col[r * W + t];
      vs[t] = val[r * W + t];
    }
#pragma unroll
    for (int t = 0; t < W; ++t) xs[t] = in[base + cs[t] * stride];
    T acc = T(0);
#pragma unroll
    for (int t = 0; t < W; ++t) {
      bool zero = false;
      if (mask_in)
        zero = dev_constrained(min, dir == 0 ? cs[t] : cx, dir == 1 ? cs[t] : cy, dir == 2 ? cs[t] : cz);
      acc += zero ? T(0) : vs[t] * xs[t];
    }
    if (accumulate) {
      if (!dev_constrained(mout, cx, cy, cz)) out[i] += acc;
    } else {
      out[i] = acc;
    }
  }
}

// the three passes of a transfer in one kernel when every direction has at most W = 3 taps per
// row (all transfers of cphMG except the finest continuous p-step): a thread per destination node
// sums the W^3 products of its three 1D rows (constrained input nodes read as zero), and adds at
// an unconstrained destination node
template <class T, int W>
__global__ void lattice_transfer_direct_kernel(const T* __restrict__ in, T* __restrict__ out, int o0, int o1, int o2,
                                               int i0, int i1, const int* __restrict__ cx, const T* __restrict__ vx,
                                               const int* __restrict__ cy, const T* __restrict__ vy,
                                               const int* __restrict__ cz, const T* __restrict__ vz,
                                               const __grid_constant__ LatticeMask min,
                                               const __grid_constant__ LatticeMask mout) {
  const int total = o0 * o1 * o2;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int x = i % o0, y = (i / o0) % o1, z = i / (o0 * o1);
    if (dev_constrained(mout, x, y, z)) continue;
    int ax[W], ay[W], az[W];
    T wx[W], wy[W], wz[W];
    bool fx[W], fy[W], fz[W];
#pragma unroll
    for (int t = 0; t < W; ++t) {
      ax[t] = cx[x * W + t];
      ay[t] = cy[y * W + t];
      az[t] = cz[z * W + t];
      wx[t] = vx[x * W + t];
      wy[t] = vy[y * W + t];
      wz[t] = vz[z * W + t];
      fx[t] = !min.periodic[0] && ((ax[t] == 0 && min.dirichlet[0]) || (ax[t] == min.n[0] - 1 && min.dirichlet[1]));
      fy[t] = !min.periodic[1] && ((ay[t] == 0 && min.dirichlet[2]) || (ay[t] == min.n[1] - 1 && min.dirichlet[3]));
      fz[t] = !min.periodic[2] && ((az[t] == 0 && min.dirichlet[4]) || (az[t] == min.n[2] - 1 && min.dirichlet[5]));
    }
    T acc = T(0);
#pragma unroll
    for (int c = 0; c < W; ++c)
#pragma unroll
      for (int b = 0; b < W; ++b) {
        T row = T(0);
        const int rbase = i0 * (ay[b] + i1 * az[c]);
#pragma unroll
        for (int a = 0; a < W; ++a) {
          const bool zero = fx[a] || fy[b] || fz[c] || (min.pin_first && ax[a] == 0 && ay[b] == 0 && az[c] == 0);
          row += zero ? T(0) : wx[a] * in[rbase + ax[a]];
        }
        acc += wy[b] * wz[c] * row;
      }
    out[i] += acc;
  }
}

// tap counts with a compiled pass
static int padded_width(int w) {
  for (int c : {2, 3, 4, 5, 6, 8, 10, 12, 17})
    if (w <= c) return c;
  EXG_CHECK(false, EXG_ERR_UNSUPPORTED, "transfer row too wide");
  return 0;
}

// c-transfer: every DG DoF reads its lattice node (K compile-time: the index splits are
// multiply-shifts)
template <class T, int K, bool SET = false>
__global__ void c_prolongate_kernel(const T* __restrict__ coarse, T* __restrict__ fine,
                                    const __grid_constant__ LatticeMask m, int N0, int N1, int N2) {
  constexpr int n = K + 1, n3 = n * n * n;
  const long long total = (long long)N0 * N1 * N2 * n3;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long c = i / n3;
    const int q = (int)(i - c * n3);
    const int cx = (int)(c % N0), cyz = (int)(c / N0), cy = cyz % N1, cz = cyz / N1;
    int g[3] = {cx * K + q % n, cy * K + (q / n) % n, cz * K + q / (n * n)};
    for (int d = 0; d < 3; ++d)
      if (m.periodic[d] && g[d] >= m.n[d]) g[d] -= m.n[d];
    const T v = dev_constrained(m, g[0], g[1], g[2]) ? T(0)
                                                      : coarse[g[0] + (long long)m.n[0] * (g[1] + (long long)m.n[1] * g[2])];
    if (SET)
      fine[i] = v;
    else
      fine[i] += v;
  }
}

// c-transfer restriction: every unconstrained lattice node sums the DG DoFs at its position
// (one cell in each direction, two at a cell vertex).  MODE 0: coarse += sum (the transfer);
// MODE 1: the continuous operator on a curved mesh, t = sum of the cell terms, src on constrained
// nodes, stored through the point epilogue; MODE 2: the diagonal (1 on constrained nodes,
// inverted when asked)
template <class T, int K, int MODE = 0>
__global__ void c_restrict_kernel(const T* __restrict__ fine, T* __restrict__ coarse,
                                  const __grid_constant__ LatticeMask m, int N0, int N1, int N2,
                                  const T* __restrict__ src = nullptr, PointEpilogue ep = PointEpilogue(),
                                  int invert = 0) {
  constexpr int n = K + 1;
  const int Nd[3] = {N0, N1, N2};
  const long long total = (long long)m.n[0] * m.n[1] * m.n[2];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int ii = (int)i;  // lattices have fewer than 2^31 nodes
    const int g[3] = {ii % m.n[0], (ii / m.n[0]) % m.n[1], ii / (m.n[0] * m.n[1])};
    if (dev_constrained(m, g[0], g[1], g[2])) {
      if (MODE == 1) epilogue_store<T>(ep, coarse, i, src, src[i]);
      if (MODE == 2) coarse[i] = T(1);
      continue;
    }
    int cell[3][2], loc[3][2], cnt[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int e = g[d] / K, l = g[d] - e * K;
      cnt[d] = 0;
      if (l != 0) {
        cell[d][0] = e;
        loc[d][0] = l;
        cnt[d] = 1;
        continue;
      }
      if (e >= 1 || m.periodic[d]) {  // left cell, its last node
        cell[d][cnt[d]] = e >= 1 ? e - 1 : Nd[d] - 1;
        loc[d][cnt[d]] = K;
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
          acc += fine[c * (n * n * n) + loc[0][cx] + n * (loc[1][cy] + n * loc[2][cz])];
        }
    if (MODE == 0) coarse[i] += acc;
    if (MODE == 1) epilogue_store<T>(ep, coarse, i, src, acc);
    if (MODE == 2) coarse[i] = invert ? (fabs((double)acc) > 1e-10 ? T(1) / acc : T(1)) : acc;
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
    // prolongation rows: fine node -> kc+1 coarse nodes of the coarse cell around it (zero taps pad
    // the row to a compiled width)
    const int w = padded_width(kc + 1);
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
      for (int j = 0; j <= kc; ++j) rows[pc[(size_t)g * w + j]].push_back({g, pv[(size_t)g * w + j]});
    int wr_d = 1;
    for (auto& r : rows) wr_d = std::max(wr_d, (int)r.size());
    wr_d = padded_width(wr_d);
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
  EXG_CHECK(total < (1LL << 31), EXG_ERR_INVALID, "lattice too large");
  LatticeMask none{};
  const int g = grid_for(total);
#define EXG_PASS(WW)                                                                                          \
  case WW:                                                                                                    \
    lattice_pass_kernel<T, WW><<<g, 256, 0, s>>>(in, out, dims_out[0], dims_out[1], dims_out[2], dir, n_in_dir, \
                                                 col, (const T*)val, min ? *min : none, min ? 1 : 0,          \
                                                 mout ? *mout : none, mout ? 1 : 0);                          \
    break;
  switch (w) {
    EXG_PASS(2)
    EXG_PASS(3)
    EXG_PASS(4)
    EXG_PASS(5)
    EXG_PASS(6)
    EXG_PASS(8)
    EXG_PASS(10)
    EXG_PASS(12)
    EXG_PASS(17)
    default:
      EXG_CHECK(false, EXG_ERR_UNSUPPORTED, "transfer row width");
  }
#undef EXG_PASS
  EXG_CUDA(cudaGetLastError());
  (void)t;
}

template <class T>
static void prolongate_t(const LatticeTransfer& t, const T* coarse, T* fine, cudaStream_t s) {
  if (t.to_dg) {
    const long long total = (long long)t.Nc[0] * t.Nc[1] * t.Nc[2] * (t.kc + 1) * (t.kc + 1) * (t.kc + 1);
    switch (t.kc) {
#define EXG_CP(KK)                                                                                          \
  case KK:                                                                                                  \
    c_prolongate_kernel<T, KK><<<grid_for(total), 256, 0, s>>>(coarse, fine, t.mc, t.Nc[0], t.Nc[1], t.Nc[2]); \
    break;
      EXG_CP(1) EXG_CP(2) EXG_CP(3) EXG_CP(4) EXG_CP(5) EXG_CP(6) EXG_CP(7) EXG_CP(8)
#undef EXG_CP
      default:
        EXG_CHECK(false, EXG_ERR_UNSUPPORTED, "continuous level degree must be 1..8");
    }
    EXG_CUDA(cudaGetLastError());
    return;
  }
  if (t.wp[0] == 2 && t.wp[1] == 2 && t.wp[2] == 2) {
    const long long total = (long long)t.mf.n[0] * t.mf.n[1] * t.mf.n[2];
    lattice_transfer_direct_kernel<T, 2><<<grid_for(total), 256, 0, s>>>(
        coarse, fine, t.mf.n[0], t.mf.n[1], t.mf.n[2], t.mc.n[0], t.mc.n[1], t.pcol[0], (const T*)t.pval[0], t.pcol[1],
        (const T*)t.pval[1], t.pcol[2], (const T*)t.pval[2], t.mc, t.mf);
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
    const int g = grid_for((long long)t.mc.n[0] * t.mc.n[1] * t.mc.n[2]);
    switch (t.kc) {
#define EXG_CR(KK)                                                                                 \
  case KK:                                                                                         \
    c_restrict_kernel<T, KK><<<g, 256, 0, s>>>(fine, coarse, t.mc, t.Nc[0], t.Nc[1], t.Nc[2]); \
    break;
      EXG_CR(1) EXG_CR(2) EXG_CR(3) EXG_CR(4) EXG_CR(5) EXG_CR(6) EXG_CR(7) EXG_CR(8)
#undef EXG_CR
      default:
        EXG_CHECK(false, EXG_ERR_UNSUPPORTED, "continuous level degree must be 1..8");
    }
    EXG_CUDA(cudaGetLastError());
    return;
  }
  if (t.wr[0] == 3 && t.wr[1] == 3 && t.wr[2] == 3) {
    const long long total = (long long)t.mc.n[0] * t.mc.n[1] * t.mc.n[2];
    lattice_transfer_direct_kernel<T, 3><<<grid_for(total), 256, 0, s>>>(
        fine, coarse, t.mc.n[0], t.mc.n[1], t.mc.n[2], t.mf.n[0], t.mf.n[1], t.rcol[0], (const T*)t.rval[0], t.rcol[1],
        (const T*)t.rval[1], t.rcol[2], (const T*)t.rval[2], t.mf, t.mc);
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

// ------------------------------------------------------------------------------------------
// curved continuous levels: the lattice and the DG layout of the same mesh and degree
// ------------------------------------------------------------------------------------------
template <class T>
static void to_dg_t(const LatticeHost& L, const T* lat, T* dg, cudaStream_t s) {
  const long long total = (long long)L.N[0] * L.N[1] * L.N[2] * (L.k + 1) * (L.k + 1) * (L.k + 1);
  switch (L.k) {
#define EXG_TD(KK)                                                                                              \
  case KK:                                                                                                      \
    c_prolongate_kernel<T, KK, true><<<grid_for(total), 256, 0, s>>>(lat, dg, L.mask, L.N[0], L.N[1], L.N[2]); \
    break;
    EXG_TD(1) EXG_TD(2) EXG_TD(3) EXG_TD(4) EXG_TD(5) EXG_TD(6) EXG_TD(7) EXG_TD(8)
#undef EXG_TD
    default:
      EXG_CHECK(false, EXG_ERR_UNSUPPORTED, "continuous level degree must be 1..8");
  }
  EXG_CUDA(cudaGetLastError());
}

template <class T, int MODE>
static void from_dg_t(const LatticeHost& L, const T* dg, const T* src, T* out, const PointEpilogue& ep, bool invert,
                      cudaStream_t s) {
  const int g = grid_for(L.size());
  switch (L.k) {
#define EXG_FD(KK)                                                                                               \
  case KK:                                                                                                       \
    c_restrict_kernel<T, KK, MODE><<<g, 256, 0, s>>>(dg, out, L.mask, L.N[0], L.N[1], L.N[2], src, ep, invert ? 1 : 0); \
    break;
    EXG_FD(1) EXG_FD(2) EXG_FD(3) EXG_FD(4) EXG_FD(5) EXG_FD(6) EXG_FD(7) EXG_FD(8)
#undef EXG_FD
    default:
      EXG_CHECK(false, EXG_ERR_UNSUPPORTED, "continuous level degree must be 1..8");
  }
  EXG_CUDA(cudaGetLastError());
}

void lattice_to_dg(const LatticeHost& L, int precision, const void* lat, void* dg, cudaStream_t s) {
  if (precision == EXG_PREC_F32)
    to_dg_t<float>(L, (const float*)lat, (float*)dg, s);
  else
    to_dg_t<double>(L, (const double*)lat, (double*)dg, s);
}

void dg_to_lattice_apply(const LatticeHost& L, int precision, const void* dg, const void* src, void* dst,
                         const PointEpilogue& ep, cudaStream_t s) {
  if (precision == EXG_PREC_F32)
    from_dg_t<float, 1>(L, (const float*)dg, (const float*)src, (float*)dst, ep, false, s);
  else
    from_dg_t<double, 1>(L, (const double*)dg, (const double*)src, (double*)dst, ep, false, s);
}

void dg_to_lattice_diagonal(const LatticeHost& L, int precision, const void* dg, void* diag, bool invert,
                            cudaStream_t s) {
  if (precision == EXG_PREC_F32)
    from_dg_t<float, 2>(L, (const float*)dg, nullptr, (float*)diag, PointEpilogue(), invert, s);
  else
    from_dg_t<double, 2>(L, (const double*)dg, nullptr, (double*)diag, PointEpilogue(), invert, s);
}

}  // namespace exg
