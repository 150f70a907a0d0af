// Element-centric SIPG Laplace apply on affine box meshes (sm_103a).
//
// On an affine box cell with QGauss(k+1) the reference's cell, face and boundary integrals
// (poisson/spatial_discretization/laplace_operator.cpp:129-265, weak_boundary_conditions.h)
// factorise exactly into
//     y = sum_d  (A_d L_d) (x) M (x) M ,
// where L_d is the 1D line operator of direction d (stiffness / h_d, SIPG flux terms of the two
// faces normal to d, penalty tau_face = max(tau-, tau+) (k+1)^2 IP), M the 1D reference mass and
// A_d the face area normal to d.  One thread block owns CPB consecutive cells; one thread owns one
// line of a cell per direction.  Every cell writes only its own DoFs (no atomics): the face fluxes
// of a cell need the neighbour's trace value and normal derivative, which the line thread reads
// from the neighbour's line (L1/L2 resident).  The 1D coefficients travel in the kernel parameter
// block (constant bank), so the FMAs read them without load instructions.
//
// Sweep schedule per cell (5 mass sweeps + 3 line operators):
//     w_x = A_x L_x u,  w_y = A_y L_y u,  w_z = A_z L_z u          (line threads, registers)
//     y   = M_z (M_y w_x + M_x w_y) + M_x M_y w_z                   (shared-memory sweeps)
#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>

#include "df64.cuh"
#include "internal.h"

namespace exg {

template <int N, class C>
struct CartCoef {
  C M[N * N];
  C B[3][N * N];
  C sdL[3][N], sdR[3][N];
  C tauA[3][64];  // A_d * tau_c * (k+1)^2 IP per cell boundary class
};

template <int N, class C>
static CartCoef<N, C> make_coef(const CartHost& h) {
  CartCoef<N, C> c;
  for (int i = 0; i < N * N; ++i) c.M[i] = coef_from_double<C>(h.M[i]);
  for (int d = 0; d < 3; ++d) {
    for (int i = 0; i < N * N; ++i) c.B[d][i] = coef_from_double<C>(h.B[d][i]);
    for (int i = 0; i < N; ++i) {
      c.sdL[d][i] = coef_from_double<C>(h.sdL[d][i]);
      c.sdR[d][i] = coef_from_double<C>(h.sdR[d][i]);
    }
    for (int cls = 0; cls < 64; ++cls) c.tauA[d][cls] = coef_from_double<C>(h.tauA[d][cls]);
  }
  return c;
}

// --------------------------------------------------------------------------------------------
// cell / face bookkeeping
// --------------------------------------------------------------------------------------------
__device__ __forceinline__ void cell_coords(const CartMesh& m, int c, int ci[3]) {
  const unsigned int uc = (unsigned int)c, n0 = (unsigned int)m.N[0], n1 = (unsigned int)m.N[1];
  const unsigned int r = uc / n0;
  ci[0] = (int)(uc - r * n0);
  ci[1] = (int)(r % n1);
  ci[2] = (int)(r / n1);
}

// boundary class of a cell (2 bits per direction: at the low / at the high non-periodic boundary);
// the penalty tau_c = surface/volume of IP::calculate_penalty_parameter
// (interior_penalty_parameter.h:45-97) depends on nothing else on a uniform box mesh
__device__ __forceinline__ int cell_class(const CartMesh& m, const int ci[3]) {
  int cls = 0;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    int lo = (ci[e] == 0 && !m.periodic[e]) ? 1 : 0;
    int hi = (ci[e] == m.N[e] - 1 && !m.periodic[e]) ? 2 : 0;
    cls |= (lo | hi) << (2 * e);
  }
  return cls;
}

__device__ __forceinline__ double cmax(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float cmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ df64 cmax(df64 a, df64 b) {
  return (a.hi > b.hi || (a.hi == b.hi && a.lo >= b.lo)) ? a : b;
}
__device__ __forceinline__ double ctwice(double a) { return 2.0 * a; }
__device__ __forceinline__ float ctwice(float a) { return 2.0f * a; }
__device__ __forceinline__ df64 ctwice(df64 a) { return df64(2.0f * a.hi, 2.0f * a.lo); }

// face f = 2d + side of cell c: neighbour index (or -1), kind (0 interior/periodic, 1 Dirichlet,
// 2 Neumann) and A_d * tau' (tau' = max(tau-, tau+) interior, 2 tau_c Dirichlet, 0 Neumann)
template <int N, class C>
__device__ __forceinline__ void face_info(const CartMesh& m, const CartCoef<N, C>& P, int c, int f, int& nb,
                                          int& kind, C& atau) {
  int ci[3];
  cell_coords(m, c, ci);
  const int d = f >> 1, side = f & 1;
  const int stride = d == 0 ? 1 : (d == 1 ? m.N[0] : m.N[0] * m.N[1]);
  const int cd = ci[d];
  const C tc = P.tauA[d][cell_class(m, ci)];
  nb = -1;
  int cn[3] = {ci[0], ci[1], ci[2]};
  if (side == 1) {
    if (cd + 1 < m.N[d]) {
      nb = c + stride;
      cn[d] = cd + 1;
    } else if (m.periodic[d]) {
      nb = c - (m.N[d] - 1) * stride;
      cn[d] = 0;
    }
  } else {
    if (cd > 0) {
      nb = c - stride;
      cn[d] = cd - 1;
    } else if (m.periodic[d]) {
      nb = c + (m.N[d] - 1) * stride;
      cn[d] = m.N[d] - 1;
    }
  }
  if (nb >= 0) {
    kind = 0;
    atau = cmax(tc, P.tauA[d][cell_class(m, cn)]);
  } else {
    kind = m.bc[f] == EXG_BC_DIRICHLET ? 1 : 2;
    atau = kind == 1 ? ctwice(tc) : C(0);
  }
}

template <int D, int N>
__device__ __forceinline__ int line_index(int i, int a, int b) {
  return D == 0 ? i + N * (a + N * b) : (D == 1 ? a + N * (i + N * b) : a + N * (b + N * i));
}

// w = A_d L_d u on the line (a, b) of direction D
template <int D, int N, class T, class C>
__device__ __forceinline__ void line_operator(const C* __restrict__ su, C* __restrict__ wout, int a, int b,
                                              const CartCoef<N, C>& P, const T* __restrict__ src,
                                              const int* nb, const int* kind, const C* atau) {
  constexpr int N3 = N * N * N;
  C u[N], w[N];
#pragma unroll
  for (int i = 0; i < N; ++i) u[i] = su[line_index<D, N>(i, a, b)];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    C acc = P.B[D][i * N] * u[0];
#pragma unroll
    for (int j = 1; j < N; ++j) acc = fmadd(P.B[D][i * N + j], u[j], acc);
    w[i] = acc;
  }
  const C tL = atau[2 * D], tR = atau[2 * D + 1];
  w[0] = fmadd(tL, u[0], w[0]);
  w[N - 1] = fmadd(tR, u[N - 1], w[N - 1]);
  // left face
  if (kind[2 * D] == 0) {
    const T* ln = src + (long long)nb[2 * D] * N3;
    C un[N];
#pragma unroll
    for (int i = 0; i < N; ++i) un[i] = load_as<C>(ln + line_index<D, N>(i, a, b));
    C ap = un[N - 1];
    C dot = P.sdR[D][0] * un[0];
#pragma unroll
    for (int i = 1; i < N; ++i) dot = fmadd(P.sdR[D][i], un[i], dot);
    C nap = neg(ap);
#pragma unroll
    for (int i = 0; i < N; ++i) w[i] = fmadd(nap, P.sdL[D][i], w[i]);
    w[0] = w[0] + fmadd(neg(tL), ap, dot);
  } else {
    C dot = P.sdL[D][0] * u[0];
#pragma unroll
    for (int i = 1; i < N; ++i) dot = fmadd(P.sdL[D][i], u[i], dot);
    C s0 = kind[2 * D] == 1 ? u[0] : neg(u[0]);
    C sd = kind[2 * D] == 1 ? dot : neg(dot);
#pragma unroll
    for (int i = 0; i < N; ++i) w[i] = fmadd(s0, P.sdL[D][i], w[i]);
    w[0] = w[0] + sd;
  }
  // right face
  if (kind[2 * D + 1] == 0) {
    const T* rn = src + (long long)nb[2 * D + 1] * N3;
    C un[N];
#pragma unroll
    for (int i = 0; i < N; ++i) un[i] = load_as<C>(rn + line_index<D, N>(i, a, b));
    C ap = un[0];
    C dot = P.sdL[D][0] * un[0];
#pragma unroll
    for (int i = 1; i < N; ++i) dot = fmadd(P.sdL[D][i], un[i], dot);
#pragma unroll
    for (int i = 0; i < N; ++i) w[i] = fmadd(ap, P.sdR[D][i], w[i]);
    w[N - 1] = w[N - 1] - fmadd(tR, ap, dot);
  } else {
    C dot = P.sdR[D][0] * u[0];
#pragma unroll
    for (int i = 1; i < N; ++i) dot = fmadd(P.sdR[D][i], u[i], dot);
    C s0 = kind[2 * D + 1] == 1 ? neg(u[N - 1]) : u[N - 1];
    C sd = kind[2 * D + 1] == 1 ? neg(dot) : dot;
#pragma unroll
    for (int i = 0; i < N; ++i) w[i] = fmadd(s0, P.sdR[D][i], w[i]);
    w[N - 1] = w[N - 1] + sd;
  }
#pragma unroll
  for (int i = 0; i < N; ++i) wout[line_index<D, N>(i, a, b)] = w[i];
}

// in-place 1D mass sweep along direction D on the line (a, b); optional second array
template <int D, int N, class C>
__device__ __forceinline__ void mass_line(C* __restrict__ x, int a, int b, const CartCoef<N, C>& P) {
  C v[N];
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = x[line_index<D, N>(i, a, b)];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    C acc = P.M[i * N] * v[0];
#pragma unroll
    for (int j = 1; j < N; ++j) acc = fmadd(P.M[i * N + j], v[j], acc);
    x[line_index<D, N>(i, a, b)] = acc;
  }
}

template <int N, int CPB, class T, class C>
__global__ void __launch_bounds__(CPB* N* N) cart_apply_kernel(const T* __restrict__ src, T* __restrict__ dst,
                                                               const __grid_constant__ CartCoef<N, C> P,
                                                               const CartMesh m) {
  constexpr int N2 = N * N, N3 = N2 * N, NT = CPB * N2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* stau = reinterpret_cast<C*>(smem_raw);             // CPB*6
  int* snb = reinterpret_cast<int*>(stau + CPB * 6);     // CPB*6
  int* skind = snb + CPB * 6;                            // CPB*6
  C* su = reinterpret_cast<C*>(smem_raw + smem_head_bytes<C>(CPB));
  C* wx = su + CPB * N3;
  C* wy = wx + CPB * N3;
  C* wz = wy + CPB * N3;

  const long long c0 = (long long)blockIdx.x * CPB;
  const T* s = src + (long long)blockIdx.y * m.n_dofs;
  T* o = dst + (long long)blockIdx.y * m.n_dofs;
  const int tid = threadIdx.x;
  const long long base = c0 * N3;
  const long long ncell_here = min((long long)CPB, m.n_cells - c0);
  const int nd = (int)(ncell_here * N3);

  for (int i = tid; i < CPB * N3; i += NT) su[i] = i < nd ? load_as<C>(s + base + i) : C(0);
  for (int t = tid; t < CPB * 6; t += NT) {  // NT < 6 CPB for k = 1
    int lc = t / 6, f = t - lc * 6;
    long long c = c0 + lc;
    int nb = -1, kind = 2;
    C at = C(0);
    if (c < m.n_cells) face_info<N, C>(m, P, (int)c, f, nb, kind, at);
    snb[t] = nb;
    skind[t] = kind;
    stau[t] = at;
  }
  __syncthreads();

  const int lc = tid / N2, l = tid - lc * N2, a = l % N, b = l / N;
  const bool active = lc < ncell_here;
  const int co = lc * N3;
  if (active) {
    line_operator<0, N, T, C>(su + co, wx + co, a, b, P, s, snb + lc * 6, skind + lc * 6, stau + lc * 6);
    line_operator<1, N, T, C>(su + co, wy + co, a, b, P, s, snb + lc * 6, skind + lc * 6, stau + lc * 6);
    line_operator<2, N, T, C>(su + co, wz + co, a, b, P, s, snb + lc * 6, skind + lc * 6, stau + lc * 6);
  }
  __syncthreads();
  if (active) {
    mass_line<1, N, C>(wx + co, a, b, P);
    mass_line<1, N, C>(wz + co, a, b, P);
  }
  __syncthreads();
  if (active) {
    mass_line<0, N, C>(wy + co, a, b, P);
    mass_line<0, N, C>(wz + co, a, b, P);
  }
  __syncthreads();
  if (active) {
    // z-line (i = a, j = b): y = M_z (wx + wy) + wz, stored straight to global memory (for a
    // fixed k the threads of a cell write N*N consecutive values)
    C v[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
      int id = line_index<2, N>(k, a, b);
      v[k] = wx[co + id] + wy[co + id];
    }
    T* oc = o + base + co;
#pragma unroll
    for (int k = 0; k < N; ++k) {
      int id = line_index<2, N>(k, a, b);
      C acc = wz[co + id];
#pragma unroll
      for (int j = 0; j < N; ++j) acc = fmadd(P.M[k * N + j], v[j], acc);
      store_as<T>(oc + id, acc);
    }
  }
}

// diagonal: sum_d diag(A_d L_d^self)[i_d] * M[i_e][i_e] * M[i_f][i_f]
// (MatrixFreeTools::compute_diagonal via operator_base.cpp:618-646; inversion per invert_diagonal.h)
template <int N, class T, class C>
__global__ void cart_diag_kernel(T* __restrict__ diag, const __grid_constant__ CartCoef<N, C> P, const CartMesh m,
                                 bool invert) {
  constexpr int N3 = N * N * N;
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= m.n_dofs) return;
  long long c = g / N3;
  int loc = (int)(g - c * N3);
  int idx[3] = {loc % N, (loc / N) % N, loc / (N * N)};
  double sum = 0.0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int i = idx[d];
    double v = coef_to_double(P.B[d][i * N + i]);
    if (i == 0) {
      int nb, kind;
      C at;
      face_info<N, C>(m, P, (int)c, 2 * d, nb, kind, at);
      v += coef_to_double(at);
      if (kind == 1) v += 2.0 * coef_to_double(P.sdL[d][0]);
      if (kind == 2) v -= 2.0 * coef_to_double(P.sdL[d][0]);
    }
    if (i == N - 1) {
      int nb, kind;
      C at;
      face_info<N, C>(m, P, (int)c, 2 * d + 1, nb, kind, at);
      v += coef_to_double(at);
      if (kind == 1) v -= 2.0 * coef_to_double(P.sdR[d][N - 1]);
      if (kind == 2) v += 2.0 * coef_to_double(P.sdR[d][N - 1]);
    }
    int e = d == 0 ? 1 : 0, f = d == 2 ? 1 : 2;
    sum += v * coef_to_double(P.M[idx[e] * N + idx[e]]) * coef_to_double(P.M[idx[f] * N + idx[f]]);
  }
  T r = (T)sum;
  if (invert) r = fabs((double)r) > 1e-10 ? (T)1 / r : (T)1;
  diag[g] = r;
}

// --------------------------------------------------------------------------------------------
// dispatch
// --------------------------------------------------------------------------------------------
template <int N>
struct CpbChoice;
template <> struct CpbChoice<2> { static constexpr int a = 16, b = 32, c = 64; };
template <> struct CpbChoice<3> { static constexpr int a = 8, b = 16, c = 32; };
template <> struct CpbChoice<4> { static constexpr int a = 4, b = 8, c = 16; };
template <> struct CpbChoice<5> { static constexpr int a = 4, b = 8, c = 16; };
template <> struct CpbChoice<6> { static constexpr int a = 2, b = 4, c = 8; };
template <> struct CpbChoice<7> { static constexpr int a = 2, b = 4, c = 8; };
template <> struct CpbChoice<8> { static constexpr int a = 1, b = 2, c = 4; };
template <> struct CpbChoice<9> { static constexpr int a = 1, b = 2, c = 4; };

template <int N, int CPB, class T, class C>
static void launch_apply(const CartHost& h, const void* src, void* dst, int n_rhs, cudaStream_t s) {
  constexpr int N3 = N * N * N;
  CartCoef<N, C> P = make_coef<N, C>(h);
  size_t smem = smem_head_bytes<C>(CPB) + 4 * (size_t)CPB * N3 * sizeof(C);
  auto kern = cart_apply_kernel<N, CPB, T, C>;
  static bool attr_set = false;
  if (!attr_set) {
    EXG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  long long blocks = (h.mesh.n_cells + CPB - 1) / CPB;
  EXG_CHECK(blocks < (1LL << 31), EXG_ERR_INVALID, "mesh too large");
  EXG_CHECK(n_rhs >= 1 && n_rhs <= 65535, EXG_ERR_INVALID, "n_rhs out of range");
  dim3 grid((unsigned)blocks, (unsigned)n_rhs);
  kern<<<grid, CPB * N * N, smem, s>>>((const T*)src, (T*)dst, P, h.mesh);
  EXG_CUDA(cudaGetLastError());
}

template <int N, class T, class C>
static void apply_n(const CartHost& h, const void* src, void* dst, int n_rhs, int cpb, cudaStream_t s) {
  if (cpb == CpbChoice<N>::a)
    launch_apply<N, CpbChoice<N>::a, T, C>(h, src, dst, n_rhs, s);
  else if (cpb == CpbChoice<N>::c)
    launch_apply<N, CpbChoice<N>::c, T, C>(h, src, dst, n_rhs, s);
  else
    launch_apply<N, CpbChoice<N>::b, T, C>(h, src, dst, n_rhs, s);
}

template <class T, class C>
static void apply_prec(const CartHost& h, const void* src, void* dst, int n_rhs, int cpb, cudaStream_t s) {
  switch (h.n) {
    case 2: apply_n<2, T, C>(h, src, dst, n_rhs, cpb, s); break;
    case 3: apply_n<3, T, C>(h, src, dst, n_rhs, cpb, s); break;
    case 4: apply_n<4, T, C>(h, src, dst, n_rhs, cpb, s); break;
    case 5: apply_n<5, T, C>(h, src, dst, n_rhs, cpb, s); break;
    case 6: apply_n<6, T, C>(h, src, dst, n_rhs, cpb, s); break;
    case 7: apply_n<7, T, C>(h, src, dst, n_rhs, cpb, s); break;
    case 8: apply_n<8, T, C>(h, src, dst, n_rhs, cpb, s); break;
    case 9: apply_n<9, T, C>(h, src, dst, n_rhs, cpb, s); break;
    default: throw Error{EXG_ERR_UNSUPPORTED, "degree must be 1..8"};
  }
}

void cart_apply(const CartHost& h, int precision, const void* src, void* dst, int n_rhs, int cpb, cudaStream_t s) {
  if (precision == EXG_PREC_F64)
    apply_prec<double, double>(h, src, dst, n_rhs, cpb, s);
  else if (precision == EXG_PREC_F32)
    apply_prec<float, float>(h, src, dst, n_rhs, cpb, s);
  else if (precision == EXG_PREC_F64E)
    apply_prec<double, df64>(h, src, dst, n_rhs, cpb, s);
  else
    throw Error{EXG_ERR_INVALID, "unknown precision"};
}

template <int N>
static std::vector<int> cpb_list() {
  return {CpbChoice<N>::a, CpbChoice<N>::b, CpbChoice<N>::c};
}

std::vector<int> cart_cpb_options(int n, int) {
  switch (n) {
    case 2: return cpb_list<2>();
    case 3: return cpb_list<3>();
    case 4: return cpb_list<4>();
    case 5: return cpb_list<5>();
    case 6: return cpb_list<6>();
    case 7: return cpb_list<7>();
    case 8: return cpb_list<8>();
    case 9: return cpb_list<9>();
  }
  return {};
}

template <int N, class T, class C>
static void diag_n(const CartHost& h, void* diag, bool invert, cudaStream_t s) {
  CartCoef<N, C> P = make_coef<N, C>(h);
  long long blocks = (h.mesh.n_dofs + 255) / 256;
  cart_diag_kernel<N, T, C><<<(unsigned)blocks, 256, 0, s>>>((T*)diag, P, h.mesh, invert);
  EXG_CUDA(cudaGetLastError());
}

template <class T, class C>
static void diag_prec(const CartHost& h, void* diag, bool invert, cudaStream_t s) {
  switch (h.n) {
    case 2: diag_n<2, T, C>(h, diag, invert, s); break;
    case 3: diag_n<3, T, C>(h, diag, invert, s); break;
    case 4: diag_n<4, T, C>(h, diag, invert, s); break;
    case 5: diag_n<5, T, C>(h, diag, invert, s); break;
    case 6: diag_n<6, T, C>(h, diag, invert, s); break;
    case 7: diag_n<7, T, C>(h, diag, invert, s); break;
    case 8: diag_n<8, T, C>(h, diag, invert, s); break;
    case 9: diag_n<9, T, C>(h, diag, invert, s); break;
    default: throw Error{EXG_ERR_UNSUPPORTED, "degree must be 1..8"};
  }
}

void cart_diagonal(const CartHost& h, int precision, void* diag, bool invert, cudaStream_t s) {
  // the diagonal is computed in double and rounded once to the storage type
  if (precision == EXG_PREC_F32)
    diag_prec<float, double>(h, diag, invert, s);
  else
    diag_prec<double, double>(h, diag, invert, s);
}

}  // namespace exg
