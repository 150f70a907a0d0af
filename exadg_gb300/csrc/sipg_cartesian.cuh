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
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>

#include "df64.cuh"
#include "epilogue.cuh"
#include "internal.h"

namespace exg {

// even-odd split of a centrosymmetric N x N matrix A (A[i][j] = A[N-1-i][N-1-j]), h = N/2:
//   e_j = x_j + x_{N-1-j}, o_j = x_j - x_{N-1-j} (j < h), middle x_h for odd N
//   y_i = ye_i + yo_i, y_{N-1-i} = ye_i - yo_i (i < h), y_h = sum_j Mid_j e_j + Mid_h x_h (odd N)
//   ye_i = sum_{j<h} E_ij e_j (+ E_ih x_h), yo_i = sum_{j<h} O_ij o_j
//   E_ij = (A_ij + A_i,N-1-j)/2, O_ij = (A_ij - A_i,N-1-j)/2
template <int N>
struct EO {
  static constexpr int h = N / 2, hm = N - N / 2;
};

template <int N, class C>
struct CartCoef {
  C M[N * N];
  C B[3][N * N];
  C sdL[3][N], sdR[3][N];
  C tauA[3][64];  // A_d * tau_c * (k+1)^2 IP per cell boundary class
  C Me[EO<N>::h * EO<N>::hm], Mo[EO<N>::h * EO<N>::h + 1], Mm[EO<N>::hm];
  C Be[3][EO<N>::h * EO<N>::hm], Bo[3][EO<N>::h * EO<N>::h + 1], Bm[3][EO<N>::hm];
};

template <int N, class C>
static void split_eo(const double* A, C* E, C* O, C* Mid) {
  constexpr int h = EO<N>::h, hm = EO<N>::hm;
  for (int i = 0; i < h; ++i) {
    for (int j = 0; j < h; ++j) {
      E[i * hm + j] = coef_from_double<C>(0.5 * (A[i * N + j] + A[i * N + N - 1 - j]));
      O[i * h + j] = coef_from_double<C>(0.5 * (A[i * N + j] - A[i * N + N - 1 - j]));
    }
    if (N % 2) E[i * hm + h] = coef_from_double<C>(A[i * N + h]);
  }
  if (N % 2) {
    for (int j = 0; j < h; ++j) Mid[j] = coef_from_double<C>(A[h * N + j]);
    Mid[h] = coef_from_double<C>(A[h * N + h]);
  }
}

// y = A x for a centrosymmetric A: plain for N <= 4 (the split saves nothing there), even-odd above
template <int N, class C>
__device__ __forceinline__ void eo_matvec(const C* __restrict__ A, const C* __restrict__ E, const C* __restrict__ O,
                                          const C* __restrict__ Mid, const C (&x)[N], C (&y)[N]) {
  if constexpr (N <= 4) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      C acc = A[i * N] * x[0];
#pragma unroll
      for (int j = 1; j < N; ++j) acc = fmadd(A[i * N + j], x[j], acc);
      y[i] = acc;
    }
    return;
  }
  constexpr int h = EO<N>::h, hm = EO<N>::hm;
  C e[h > 0 ? h : 1], o[h > 0 ? h : 1];
#pragma unroll
  for (int j = 0; j < h; ++j) {
    e[j] = x[j] + x[N - 1 - j];
    o[j] = x[j] - x[N - 1 - j];
  }
#pragma unroll
  for (int i = 0; i < h; ++i) {
    C ye = E[i * hm] * e[0];
#pragma unroll
    for (int j = 1; j < h; ++j) ye = fmadd(E[i * hm + j], e[j], ye);
    if (N % 2) ye = fmadd(E[i * hm + h], x[h], ye);
    C yo = O[i * h] * o[0];
#pragma unroll
    for (int j = 1; j < h; ++j) yo = fmadd(O[i * h + j], o[j], yo);
    y[i] = ye + yo;
    y[N - 1 - i] = ye - yo;
  }
  if (N % 2) {
    C ym = Mid[h] * x[h];
#pragma unroll
    for (int j = 0; j < h; ++j) ym = fmadd(Mid[j], e[j], ym);
    y[h] = ym;
  }
}

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
    split_eo<N, C>(h.B[d], c.Be[d], c.Bo[d], c.Bm[d]);
  }
  split_eo<N, C>(h.M, c.Me, c.Mo, c.Mm);
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
  // direction-d quantities through selects: runtime indices into small arrays would live in
  // local memory
  const int stride = d == 0 ? 1 : (d == 1 ? m.N[0] : m.N[0] * m.N[1]);
  const int cd = d == 0 ? ci[0] : (d == 1 ? ci[1] : ci[2]);
  const int Nd = d == 0 ? m.N[0] : (d == 1 ? m.N[1] : m.N[2]);
  const int per = d == 0 ? m.periodic[0] : (d == 1 ? m.periodic[1] : m.periodic[2]);
  const C tc = P.tauA[d][cell_class(m, ci)];
  nb = -1;
  int cdn = cd;
  if (side == 1) {
    if (cd + 1 < Nd) {
      nb = c + stride;
      cdn = cd + 1;
    } else if (per) {
      nb = c - (Nd - 1) * stride;
      cdn = 0;
    }
  } else {
    if (cd > 0) {
      nb = c - stride;
      cdn = cd - 1;
    } else if (per) {
      nb = c + (Nd - 1) * stride;
      cdn = Nd - 1;
    }
  }
  const int cn[3] = {d == 0 ? cdn : ci[0], d == 1 ? cdn : ci[1], d == 2 ? cdn : ci[2]};
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
  eo_matvec<N, C>(P.B[D], P.Be[D], P.Bo[D], P.Bm[D], u, w);
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
  C v[N], r[N];
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = x[line_index<D, N>(i, a, b)];
  eo_matvec<N, C>(P.M, P.Me, P.Mo, P.Mm, v, r);
#pragma unroll
  for (int i = 0; i < N; ++i) x[line_index<D, N>(i, a, b)] = r[i];
}

template <int N, int CPB, class T, class C>
__global__ void __launch_bounds__(CPB* N* N) cart_apply_kernel(const T* __restrict__ src, T* __restrict__ dst,
                                                               const __grid_constant__ CartCoef<N, C> P,
                                                               const __grid_constant__ CartMesh m, const PointEpilogue ep) {
  constexpr int N2 = N * N, N3 = N2 * N, NT = CPB * N2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* stau = reinterpret_cast<C*>(smem_raw);             // CPB*6
  int* snb = reinterpret_cast<int*>(stau + CPB * 6);     // CPB*6
  int* skind = snb + CPB * 6;                            // CPB*6
  C* su = reinterpret_cast<C*>(smem_raw + smem_head_bytes<C>(CPB));
  C* wx = su + CPB * N3;
  C* wy = wx + CPB * N3;
  C* wz = wy + CPB * N3;

  const long long c0 = m.cell_begin + (long long)blockIdx.x * CPB;
  const T* s = src + (long long)blockIdx.y * m.n_dofs;
  T* o = dst + (long long)blockIdx.y * m.n_dofs;
  const int tid = threadIdx.x;
  const long long base = c0 * N3;
  const long long ncell_here = min((long long)CPB, m.cell_end - c0);
  const int nd = (int)(ncell_here * N3);

  for (int i = tid; i < CPB * N3; i += NT) su[i] = i < nd ? load_as<C>(s + base + i) : C(0);
  for (int t = tid; t < CPB * 6; t += NT) {  // NT < 6 CPB for k = 1
    int lc = t / 6, f = t - lc * 6;
    long long c = c0 + lc;
    int nb = -1, kind = 2;
    C at = C(0);
    if (c < m.cell_end) face_info<N, C>(m, P, (int)c, f, nb, kind, at);
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
    C r[N];
    eo_matvec<N, C>(P.M, P.Me, P.Mo, P.Mm, v, r);
#pragma unroll
    for (int k = 0; k < N; ++k) {
      int id = line_index<2, N>(k, a, b);
      epilogue_store<T>(ep, o, base + co + id, s, to_storage<T>(r[k] + wz[co + id]));
    }
  }
}

// ------------------------------------------------------------------------------------------------
// Brick variant: a block owns BX x BY x BZ cells; their data and the six face-halo layers of
// neighbour cells are staged in shared memory with one coalesced load per cell (each cell is a
// contiguous run of N^3 values), converted once to the compute type.  Neighbour lines are then
// read from shared memory.  Partial bricks at the end of a direction are handled by taking the
// halo of a direction from the first / last active cell of the brick along it.
// ------------------------------------------------------------------------------------------------
template <int BX, int BY, int BZ>
struct Brick {
  static constexpr int NOWN = BX * BY * BZ;
  static constexpr int NHX = BY * BZ, NHY = BX * BZ, NHZ = BX * BY;
  static constexpr int NSLOT = NOWN + 2 * (NHX + NHY + NHZ);
  __device__ static int own(int lx, int ly, int lz) { return lx + BX * (ly + BY * lz); }
  __device__ static int halo(int d, int side, int lx, int ly, int lz) {
    if (d == 0) return NOWN + side * NHX + (ly + BY * lz);
    if (d == 1) return NOWN + 2 * NHX + side * NHY + (lx + BX * lz);
    return NOWN + 2 * NHX + 2 * NHY + side * NHZ + (lx + BX * ly);
  }
};

// w = A_d L_d u on the line (a, b) of direction D; neighbour cells in shared memory (nullptr at a
// physical boundary)
template <int D, int N, class C>
__device__ __forceinline__ void line_operator_s(const C* __restrict__ su, C* __restrict__ wout, int a, int b,
                                                const CartCoef<N, C>& P, const C* nbL, const C* nbR, int kL, int kR,
                                                C tL, C tR) {
  C u[N], w[N];
#pragma unroll
  for (int i = 0; i < N; ++i) u[i] = su[line_index<D, N>(i, a, b)];
  eo_matvec<N, C>(P.B[D], P.Be[D], P.Bo[D], P.Bm[D], u, w);
  w[0] = fmadd(tL, u[0], w[0]);
  w[N - 1] = fmadd(tR, u[N - 1], w[N - 1]);
  if (kL == 0) {
    C un[N];
#pragma unroll
    for (int i = 0; i < N; ++i) un[i] = nbL[line_index<D, N>(i, a, b)];
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
    C s0 = kL == 1 ? u[0] : neg(u[0]);
    C sd = kL == 1 ? dot : neg(dot);
#pragma unroll
    for (int i = 0; i < N; ++i) w[i] = fmadd(s0, P.sdL[D][i], w[i]);
    w[0] = w[0] + sd;
  }
  if (kR == 0) {
    C un[N];
#pragma unroll
    for (int i = 0; i < N; ++i) un[i] = nbR[line_index<D, N>(i, a, b)];
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
    C s0 = kR == 1 ? neg(u[N - 1]) : u[N - 1];
    C sd = kR == 1 ? neg(dot) : dot;
#pragma unroll
    for (int i = 0; i < N; ++i) w[i] = fmadd(s0, P.sdR[D][i], w[i]);
    w[N - 1] = w[N - 1] + sd;
  }
#pragma unroll
  for (int i = 0; i < N; ++i) wout[line_index<D, N>(i, a, b)] = w[i];
}

// shared-memory head of the brick kernel: slot base offsets (8-byte, first so that they are 8-byte
// aligned), then per own cell and face the penalty, neighbour slot and kind; rounded to 16 bytes
template <class C>
__host__ __device__ constexpr size_t brick_head_bytes(int nown, int nslot) {
  return ((size_t)nslot * sizeof(long long) + (size_t)nown * 6 * (sizeof(C) + 2 * sizeof(int)) + 15) / 16 * 16;
}

template <int N, int BX, int BY, int BZ, class T, class C>
__global__ void __launch_bounds__(BX* BY* BZ* N* N)
    cart_brick_kernel(const T* __restrict__ src, T* __restrict__ dst, const __grid_constant__ CartCoef<N, C> P,
                      const __grid_constant__ CartMesh m, int nbx, int nby, const PointEpilogue ep) {
  using B = Brick<BX, BY, BZ>;
  constexpr int N2 = N * N, N3 = N2 * N, NT = B::NOWN * N2;
  static_assert(NT >= 32, "brick needs at least one full warp");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  long long* sbase = reinterpret_cast<long long*>(smem_raw);  // NSLOT global base offsets (or -1)
  C* stau = reinterpret_cast<C*>(sbase + B::NSLOT);              // NOWN*6
  int* sslot = reinterpret_cast<int*>(stau + B::NOWN * 6);       // NOWN*6 neighbour slot or -1
  int* skind = sslot + B::NOWN * 6;                              // NOWN*6
  C* su = reinterpret_cast<C*>(smem_raw + brick_head_bytes<C>(B::NOWN, B::NSLOT));  // NSLOT*N3
  C* wx = su + B::NSLOT * N3;
  C* wy = wx + B::NOWN * N3;
  C* wz = wy + B::NOWN * N3;

  const int tid = threadIdx.x;
  const int bidx = blockIdx.x;
  const int bxi = bidx % nbx, byi = (bidx / nbx) % nby, bzi = bidx / (nbx * nby);
  const int x0[3] = {bxi * BX, byi * BY, bzi * BZ};
  const int bdim[3] = {BX, BY, BZ};
  int last[3];
#pragma unroll
  for (int e = 0; e < 3; ++e) last[e] = min(bdim[e], m.N[e] - x0[e]) - 1;
  const T* s = src + (long long)blockIdx.y * m.n_dofs;
  T* o = dst + (long long)blockIdx.y * m.n_dofs;

  // 1. stage own cells and face halos.  First the global base offset of every slot (or -1), then a
  // flattened copy in which every thread keeps four independent loads in flight.
  for (int slot = tid; slot < B::NSLOT; slot += NT) {
    int g[3] = {-1, -1, -1};
    bool ok = true;
    if (slot < B::NOWN) {
      int l[3] = {slot % BX, (slot / BX) % BY, slot / (BX * BY)};
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        g[e] = x0[e] + l[e];
        ok = ok && l[e] <= last[e];
      }
    } else {
      int r = slot - B::NOWN, d, side, p, q;
      if (r < 2 * B::NHX) {
        d = 0; side = r / B::NHX; r %= B::NHX; p = r % BY; q = r / BY;
        g[1] = x0[1] + p; g[2] = x0[2] + q; ok = p <= last[1] && q <= last[2];
      } else if (r < 2 * B::NHX + 2 * B::NHY) {
        r -= 2 * B::NHX;
        d = 1; side = r / B::NHY; r %= B::NHY; p = r % BX; q = r / BX;
        g[0] = x0[0] + p; g[2] = x0[2] + q; ok = p <= last[0] && q <= last[2];
      } else {
        r -= 2 * B::NHX + 2 * B::NHY;
        d = 2; side = r / B::NHZ; r %= B::NHZ; p = r % BX; q = r / BX;
        g[0] = x0[0] + p; g[1] = x0[1] + q; ok = p <= last[0] && q <= last[1];
      }
      int gd = side ? x0[d] + last[d] + 1 : x0[d] - 1;
      if (gd < 0 || gd >= m.N[d]) {
        if (m.periodic[d])
          gd = gd < 0 ? gd + m.N[d] : gd - m.N[d];
        else
          ok = false;
      }
      g[d] = gd;
    }
    sbase[slot] = ok ? ((long long)g[0] + (long long)m.N[0] * ((long long)g[1] + (long long)m.N[1] * g[2])) * N3 : -1;
  }
  __syncthreads();
  {
    // one full warp per slot; lane j loads elements j, j+32, ... of the cell, all loads before stores
    constexpr int PER = (N3 + 31) / 32;
    const int warp = tid >> 5, lane = tid & 31, nwarps = NT >> 5;
    for (int slot = warp; warp < nwarps && slot < B::NSLOT; slot += nwarps) {
      const long long bse = sbase[slot];
      C v[PER];
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int j = lane + 32 * q;
        v[q] = (bse >= 0 && j < N3) ? load_as<C>(s + bse + j) : C(0);
      }
      C* dstc = su + slot * N3;
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int j = lane + 32 * q;
        if (j < N3) dstc[j] = v[q];
      }
    }
  }
  // 2. face data of the own cells
  for (int t = tid; t < B::NOWN * 6; t += NT) {
    int lc = t / 6, f = t - lc * 6;
    int l[3] = {lc % BX, (lc / BX) % BY, lc / (BX * BY)};
    bool active = l[0] <= last[0] && l[1] <= last[1] && l[2] <= last[2];
    int nb = -1, kind = 2, slot = -1;
    C at = C(0);
    if (active) {
      int c = (x0[0] + l[0]) + m.N[0] * ((x0[1] + l[1]) + m.N[1] * (x0[2] + l[2]));
      face_info<N, C>(m, P, c, f, nb, kind, at);
      if (kind == 0) {
        int d = f >> 1, side = f & 1;
        int ln[3] = {l[0], l[1], l[2]};
        if (side == 1 && l[d] < last[d]) {
          ln[d] += 1;
          slot = B::own(ln[0], ln[1], ln[2]);
        } else if (side == 0 && l[d] > 0) {
          ln[d] -= 1;
          slot = B::own(ln[0], ln[1], ln[2]);
        } else {
          slot = B::halo(d, side, l[0], l[1], l[2]);
        }
      }
    }
    sslot[t] = slot;
    skind[t] = kind;
    stau[t] = at;
  }
  __syncthreads();

  const int lc = tid / N2, li = tid - lc * N2, a = li % N, b = li / N;
  const int lx = lc % BX, ly = (lc / BX) % BY, lz = lc / (BX * BY);
  const bool active = lx <= last[0] && ly <= last[1] && lz <= last[2];
  const int co = lc * N3;
  const int* ns = sslot + lc * 6;
  const int* nk = skind + lc * 6;
  const C* nt = stau + lc * 6;
  if (active) {
    const C* U = su + co;
    line_operator_s<0, N, C>(U, wx + co, a, b, P, ns[0] >= 0 ? su + ns[0] * N3 : nullptr,
                             ns[1] >= 0 ? su + ns[1] * N3 : nullptr, nk[0], nk[1], nt[0], nt[1]);
    line_operator_s<1, N, C>(U, wy + co, a, b, P, ns[2] >= 0 ? su + ns[2] * N3 : nullptr,
                             ns[3] >= 0 ? su + ns[3] * N3 : nullptr, nk[2], nk[3], nt[2], nt[3]);
    line_operator_s<2, N, C>(U, wz + co, a, b, P, ns[4] >= 0 ? su + ns[4] * N3 : nullptr,
                             ns[5] >= 0 ? su + ns[5] * N3 : nullptr, nk[4], nk[5], nt[4], nt[5]);
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
    C v[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
      int id = line_index<2, N>(k, a, b);
      v[k] = wx[co + id] + wy[co + id];
    }
    const long long gc = (long long)(x0[0] + lx) + (long long)m.N[0] * ((x0[1] + ly) + (long long)m.N[1] * (x0[2] + lz));
    C r[N];
    eo_matvec<N, C>(P.M, P.Me, P.Mo, P.Mm, v, r);
#pragma unroll
    for (int k = 0; k < N; ++k) {
      int id = line_index<2, N>(k, a, b);
      epilogue_store<T>(ep, o, gc * N3 + id, s, to_storage<T>(r[k] + wz[co + id]));
    }
  }
}

// diagonal: sum_d diag(A_d L_d^self)[i_d] * M[i_e][i_e] * M[i_f][i_f]
// (MatrixFreeTools::compute_diagonal via operator_base.cpp:618-646; inversion per invert_diagonal.h)
template <int N, class T, class C>
__global__ void cart_diag_kernel(T* __restrict__ diag, const __grid_constant__ CartCoef<N, C> P,
                                 const __grid_constant__ CartMesh m,
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
static void launch_apply(const CartHost& h, const void* src, void* dst, int n_rhs, cudaStream_t s,
                         const PointEpilogue& ep) {
  constexpr int N3 = N * N * N;
  CartCoef<N, C> P = make_coef<N, C>(h);
  size_t smem = smem_head_bytes<C>(CPB) + 4 * (size_t)CPB * N3 * sizeof(C);
  auto kern = cart_apply_kernel<N, CPB, T, C>;
  ensure_smem_attr((const void*)kern, (int)smem);
  long long blocks = (h.mesh.cell_end - h.mesh.cell_begin + CPB - 1) / CPB;
  EXG_CHECK(blocks < (1LL << 31), EXG_ERR_INVALID, "mesh too large");
  EXG_CHECK(n_rhs >= 1 && n_rhs <= 65535, EXG_ERR_INVALID, "n_rhs out of range");
  dim3 grid((unsigned)blocks, (unsigned)n_rhs);
  kern<<<grid, CPB * N * N, smem, s>>>((const T*)src, (T*)dst, P, h.mesh, ep);
  EXG_CUDA(cudaGetLastError());
}

template <int N, int BX, int BY, int BZ, class T, class C>
static void launch_brick(const CartHost& h, const void* src, void* dst, int n_rhs, cudaStream_t s,
                         const PointEpilogue& ep) {
  using Bk = Brick<BX, BY, BZ>;
  constexpr int N3 = N * N * N;
  CartCoef<N, C> P = make_coef<N, C>(h);
  size_t smem = brick_head_bytes<C>(Bk::NOWN, Bk::NSLOT) + ((size_t)Bk::NSLOT + 3 * Bk::NOWN) * N3 * sizeof(C);
  auto kern = cart_brick_kernel<N, BX, BY, BZ, T, C>;
  EXG_CHECK(smem <= 227 * 1024, EXG_ERR_UNSUPPORTED, "brick too large for shared memory");
  ensure_smem_attr((const void*)kern, (int)smem);
  int nb[3] = {(h.mesh.N[0] + BX - 1) / BX, (h.mesh.N[1] + BY - 1) / BY, (h.mesh.N[2] + BZ - 1) / BZ};
  long long blocks = (long long)nb[0] * nb[1] * nb[2];
  EXG_CHECK(blocks < (1LL << 31), EXG_ERR_INVALID, "mesh too large");
  EXG_CHECK(n_rhs >= 1 && n_rhs <= 65535, EXG_ERR_INVALID, "n_rhs out of range");
  dim3 grid((unsigned)blocks, (unsigned)n_rhs);
  kern<<<grid, Bk::NOWN * N * N, smem, s>>>((const T*)src, (T*)dst, P, h.mesh, nb[0], nb[1], ep);
  EXG_CUDA(cudaGetLastError());
}

// brick shapes per degree: -1 = BrickA, -2 = BrickB
template <int N> struct BrickChoice;
template <> struct BrickChoice<2> { static constexpr int ax = 4, ay = 4, az = 4, bx = 4, by = 4, bz = 2; };
template <> struct BrickChoice<3> { static constexpr int ax = 4, ay = 2, az = 2, bx = 4, by = 4, bz = 2; };
template <> struct BrickChoice<4> { static constexpr int ax = 2, ay = 2, az = 2, bx = 4, by = 2, bz = 2; };
template <> struct BrickChoice<5> { static constexpr int ax = 2, ay = 2, az = 2, bx = 4, by = 2, bz = 1; };
template <> struct BrickChoice<6> { static constexpr int ax = 2, ay = 2, az = 1, bx = 2, by = 2, bz = 2; };
template <> struct BrickChoice<7> { static constexpr int ax = 2, ay = 1, az = 1, bx = 2, by = 2, bz = 1; };
template <> struct BrickChoice<8> { static constexpr int ax = 2, ay = 1, az = 1, bx = 2, by = 2, bz = 1; };
template <> struct BrickChoice<9> { static constexpr int ax = 1, ay = 1, az = 1, bx = 2, by = 1, bz = 1; };

template <int N, class T, class C>
static void apply_n(const CartHost& h, const void* src, void* dst, int n_rhs, int cpb, cudaStream_t s,
                    const PointEpilogue& ep) {
  using BC = BrickChoice<N>;
  // bricks cover the whole mesh; a launch over a cell range uses the row kernel
  if (cpb < 0 && (h.mesh.cell_begin != 0 || h.mesh.cell_end != h.mesh.n_cells)) cpb = CpbChoice<N>::b;
  if (cpb == -1)
    launch_brick<N, BC::ax, BC::ay, BC::az, T, C>(h, src, dst, n_rhs, s, ep);
  else if (cpb == -2)
    launch_brick<N, BC::bx, BC::by, BC::bz, T, C>(h, src, dst, n_rhs, s, ep);
  else if (cpb == CpbChoice<N>::a)
    launch_apply<N, CpbChoice<N>::a, T, C>(h, src, dst, n_rhs, s, ep);
  else if (cpb == CpbChoice<N>::c)
    launch_apply<N, CpbChoice<N>::c, T, C>(h, src, dst, n_rhs, s, ep);
  else
    launch_apply<N, CpbChoice<N>::b, T, C>(h, src, dst, n_rhs, s, ep);
}

template <class T, class C>
static void apply_prec(const CartHost& h, const void* src, void* dst, int n_rhs, int cpb, cudaStream_t s,
                       const PointEpilogue& ep) {
  switch (h.n) {
    case 2: apply_n<2, T, C>(h, src, dst, n_rhs, cpb, s, ep); break;
    case 3: apply_n<3, T, C>(h, src, dst, n_rhs, cpb, s, ep); break;
    case 4: apply_n<4, T, C>(h, src, dst, n_rhs, cpb, s, ep); break;
    case 5: apply_n<5, T, C>(h, src, dst, n_rhs, cpb, s, ep); break;
    case 6: apply_n<6, T, C>(h, src, dst, n_rhs, cpb, s, ep); break;
    case 7: apply_n<7, T, C>(h, src, dst, n_rhs, cpb, s, ep); break;
    case 8: apply_n<8, T, C>(h, src, dst, n_rhs, cpb, s, ep); break;
    case 9: apply_n<9, T, C>(h, src, dst, n_rhs, cpb, s, ep); break;
    default: throw Error{EXG_ERR_UNSUPPORTED, "degree must be 1..8"};
  }
}


}  // namespace exg
