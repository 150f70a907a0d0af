// SIPG Laplace operator on curved (MappingQ) hex meshes, plus the geometry setup, right-hand side,
// diagonal and quadrature points shared by all meshes.
//
// Geometry: the mapping interpolates the chart manifold (DeformedCubeManifold::push_forward,
// grid/deformed_cube_manifold.h:47-59) at the Gauss-Lobatto support points of degree m in every
// cell, as MappingQ(m) does with a chart manifold.  A setup kernel evaluates x, J at the cell and
// face quadrature points (QGauss(k+1)) in FP64 and stores, per cell:
//   cell  q : G = JxW J^{-1} J^{-T} (6 values)            -- do_cell_integral, laplace_operator.cpp:129-137
//   face  q : a_own = J_own^{-1} n-, a_nb = J_nb^{-1} n-, JxW-   -- do_face_integral :139-163
// with n- / JxW- taken from the '-' (interior) side of every face as deal.II's FEFaceEvaluation does.
//
// Apply kernel: element-centric; CPB cells per block, one thread per line of a cell for the
// volume sweeps and one thread per face point for the face terms.  No atomics.
#include <cuda_runtime.h>

#include <cmath>

#include "df64.cuh"
#include "epilogue.cuh"
#include "general.h"
#include "internal.h"

namespace exg {

// ------------------------------------------------------------------------------------------------
// geometry setup (FP64)
// ------------------------------------------------------------------------------------------------
struct MapParams {
  int m1;  // mapping nodes per direction
  double nodes[12];
  double gq[10], gw[10];
  int nq;
  double lo[3], h[3];
  double amp, left, right;
  int freq;
  int N[3];
  int periodic[3];
};

__device__ double lag(const double* z, int n, int i, double x) {
  double v = 1.0;
  for (int j = 0; j < n; ++j)
    if (j != i) v *= (x - z[j]) / (z[i] - z[j]);
  return v;
}
__device__ double lag_d(const double* z, int n, int i, double x) {
  double s = 0.0;
  for (int m = 0; m < n; ++m) {
    if (m == i) continue;
    double t = 1.0 / (z[i] - z[m]);
    for (int j = 0; j < n; ++j)
      if (j != i && j != m) t *= (x - z[j]) / (z[i] - z[j]);
    s += t;
  }
  return s;
}

// x(xi) and J(xi) of cell ci from the manifold interpolated at the (m+1)^3 mapping support points
// (MappingQ of the deformed cube).  The deformation is separable, p_e(X) = X_e + amp prod_d S(X_d)
// with S(t) = sin(freq pi (t - left) / (right - left)), so the interpolant factorises: with the 1D
// Lagrange weights v_d(xi_d) of the support nodes, x_e = sum_a v_e,a X_e(a) + amp I_0 I_1 I_2 and
// I_d = sum_a v_d,a S(X_d(a)) (the weights sum to one), and the Jacobian follows from the 1D
// derivative weights.  3 (m+1) sines per point instead of 3 (m+1)^3.
__device__ void map_eval(const MapParams& P, const int ci[3], const double xi[3], double x[3], double J[3][3]) {
  double I[3], dI[3], A[3], dA[3];
  for (int d = 0; d < 3; ++d) {
    double si = 0, dsi = 0, ai = 0, dai = 0;
    for (int k = 0; k < P.m1; ++k) {
      const double v = lag(P.nodes, P.m1, k, xi[d]), dv = lag_d(P.nodes, P.m1, k, xi[d]);
      const double X = P.lo[d] + (ci[d] + P.nodes[k]) * P.h[d];
      const double S = P.amp != 0.0 ? sin(P.freq * M_PI * (X - P.left) / (P.right - P.left)) : 0.0;
      si += v * S;
      dsi += dv * S;
      ai += v * X;
      dai += dv * X;
    }
    I[d] = si;
    dI[d] = dsi;
    A[d] = ai;
    dA[d] = dai;
  }
  const double s = P.amp * I[0] * I[1] * I[2];
  const double g[3] = {P.amp * dI[0] * I[1] * I[2], P.amp * I[0] * dI[1] * I[2], P.amp * I[0] * I[1] * dI[2]};
  for (int e = 0; e < 3; ++e) {
    x[e] = A[e] + s;
    for (int d = 0; d < 3; ++d) J[e][d] = (e == d ? dA[d] : 0.0) + g[d];
  }
}

__device__ double inv3(const double J[3][3], double Ji[3][3]) {
  double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
               J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  double id = 1.0 / det;
  Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
  Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  return det;
}

__device__ __forceinline__ void tang(int d, int& t1, int& t2) {
  t1 = d == 0 ? 1 : 0;
  t2 = d == 2 ? 1 : 2;
}

__device__ __forceinline__ void coords3(const int N[3], long long c, int ci[3]) {
  ci[0] = (int)(c % N[0]);
  long long r = c / N[0];
  ci[1] = (int)(r % N[1]);
  ci[2] = (int)(r / N[1]);
}

__device__ long long neighbor_of(const MapParams& P, long long c, int f) {
  int ci[3];
  coords3(P.N, c, ci);
  int d = f / 2, side = f % 2;
  ci[d] += side ? 1 : -1;
  if (ci[d] < 0 || ci[d] >= P.N[d]) {
    if (!P.periodic[d]) return -1;
    ci[d] = (ci[d] + P.N[d]) % P.N[d];
  }
  return ci[0] + (long long)P.N[0] * (ci[1] + (long long)P.N[1] * ci[2]);
}

// raw data per point: cell q -> [G(6), JxW, x(3)]; face q -> [Jinv(9), n(3), JxW, x(3)]
__global__ void geom_raw_kernel(MapParams P, long long n_cells, double* __restrict__ cell_raw,
                                double* __restrict__ face_raw) {
  const int nq = P.nq, nq3 = nq * nq * nq, nq2 = nq * nq, per = nq3 + 6 * nq2;
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_cells * per) return;
  long long c = g / per;
  int p = (int)(g - c * per);
  int ci[3];
  coords3(P.N, c, ci);
  double xi[3], x[3], J[3][3], Ji[3][3];
  if (p < nq3) {
    int q0 = p % nq, q1 = (p / nq) % nq, q2 = p / nq2;
    xi[0] = P.gq[q0];
    xi[1] = P.gq[q1];
    xi[2] = P.gq[q2];
    map_eval(P, ci, xi, x, J);
    double det = inv3(J, Ji);
    double JxW = fabs(det) * P.gw[q0] * P.gw[q1] * P.gw[q2];
    double* o = cell_raw + (c * nq3 + p) * 10;
    int k = 0;
    for (int a = 0; a < 3; ++a)
      for (int b = a; b < 3; ++b) {
        double s = 0;
        for (int j = 0; j < 3; ++j) s += Ji[a][j] * Ji[b][j];
        o[k++] = s * JxW;
      }
    o[6] = JxW;
    o[7] = x[0];
    o[8] = x[1];
    o[9] = x[2];
  } else {
    int r = p - nq3;
    int f = r / nq2, qq = r - f * nq2;
    int d = f / 2, side = f % 2, t1, t2;
    tang(d, t1, t2);
    int a = qq % nq, b = qq / nq;
    xi[d] = side;
    xi[t1] = P.gq[a];
    xi[t2] = P.gq[b];
    map_eval(P, ci, xi, x, J);
    double det = inv3(J, Ji);
    double sg = side ? 1.0 : -1.0, n[3], nn = 0;
    for (int j = 0; j < 3; ++j) {
      n[j] = sg * Ji[d][j];
      nn += n[j] * n[j];
    }
    nn = sqrt(nn);
    double* o = face_raw + ((c * 6 + f) * nq2 + qq) * 16;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) o[i * 3 + j] = Ji[i][j];
    for (int j = 0; j < 3; ++j) o[9 + j] = n[j] / nn;
    o[12] = fabs(det) * nn * P.gw[a] * P.gw[b];
    o[13] = x[0];
    o[14] = x[1];
    o[15] = x[2];
  }
}

// penalty per cell: sum_f w_f |f| / |K|  (interior_penalty_parameter.h:45-97)
__global__ void geom_tau_kernel(MapParams P, long long n_cells, const double* __restrict__ cell_raw,
                                const double* __restrict__ face_raw, double* __restrict__ tau) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  const int nq = P.nq, nq3 = nq * nq * nq, nq2 = nq * nq;
  double vol = 0, surf = 0;
  for (int q = 0; q < nq3; ++q) vol += cell_raw[(c * nq3 + q) * 10 + 6];
  for (int f = 0; f < 6; ++f) {
    double w = neighbor_of(P, c, f) < 0 ? 1.0 : 0.5;
    for (int q = 0; q < nq2; ++q) surf += w * face_raw[((c * 6 + f) * nq2 + q) * 16 + 12];
  }
  tau[c] = surf / vol;
}

// final per-cell data in precision T: cell G (6) and face [a_own(3), a_nb(3), JxW] (7), the
// '-' side supplying n and JxW; face penalty / kind per cell-face
template <class T>
__global__ void geom_final_kernel(MapParams P, long long n_cells, double factor, const int* __restrict__ bc,
                                  const double* __restrict__ cell_raw, const double* __restrict__ face_raw,
                                  const double* __restrict__ tau, T* __restrict__ cellG, T* __restrict__ face,
                                  T* __restrict__ ftau, long long* __restrict__ fnb) {
  const int nq = P.nq, nq3 = nq * nq * nq, nq2 = nq * nq, per = nq3 + 6 * nq2;
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_cells * per) return;
  long long c = g / per;
  int p = (int)(g - c * per);
  if (p < nq3) {
    const double* r = cell_raw + (c * nq3 + p) * 10;
    for (int k = 0; k < 6; ++k) cellG[(c * nq3 + p) * 6 + k] = coef_from_double<T>(r[k]);
    return;
  }
  int rr = p - nq3;
  int f = rr / nq2, q = rr - f * nq2;
  int d = f / 2, side = f % 2;
  long long nb = neighbor_of(P, c, f);
  const double* ro = face_raw + ((c * 6 + f) * nq2 + q) * 16;
  const double* rm = ro;
  const double* rn = nullptr;
  if (nb >= 0) {
    rn = face_raw + ((nb * 6 + (2 * d + 1 - side)) * nq2 + q) * 16;
    if (side == 0) rm = rn;
  }
  const double* nrm = rm + 9;
  T* o = face + ((c * 6 + f) * nq2 + q) * 7;
  for (int i = 0; i < 3; ++i) {
    o[i] = coef_from_double<T>(ro[i * 3 + 0] * nrm[0] + ro[i * 3 + 1] * nrm[1] + ro[i * 3 + 2] * nrm[2]);
    o[3 + i] = coef_from_double<T>(rn ? rn[i * 3 + 0] * nrm[0] + rn[i * 3 + 1] * nrm[1] + rn[i * 3 + 2] * nrm[2] : 0.0);
  }
  o[6] = coef_from_double<T>(rm[12]);
  if (q == 0) {
    double t = nb >= 0 ? fmax(tau[c], tau[nb]) * factor : tau[c] * factor;
    ftau[c * 6 + f] = coef_from_double<T>(t);
    // encoding: >= 0 neighbour cell; -1 Dirichlet; -2 Neumann
    fnb[c * 6 + f] = nb >= 0 ? nb : (bc[f] == EXG_BC_DIRICHLET ? -1 : -2);
  }
}

static MapParams map_params(const MeshInfo& m, const FE1D& fe) {
  MapParams P{};
  int md = m.d.mapping_degree < 1 ? 1 : m.d.mapping_degree;
  EXG_CHECK(md <= 10, EXG_ERR_UNSUPPORTED, "mapping degree must be <= 10");
  std::vector<double> z = gauss_lobatto(md + 1);
  P.m1 = md + 1;
  for (int i = 0; i < P.m1; ++i) P.nodes[i] = z[i];
  P.nq = fe.nq;
  for (int i = 0; i < fe.nq; ++i) {
    P.gq[i] = fe.gq[i];
    P.gw[i] = fe.gw[i];
  }
  for (int e = 0; e < 3; ++e) {
    P.lo[e] = m.d.lo[e];
    P.h[e] = m.h[e];
    P.N[e] = m.N[e];
    P.periodic[e] = m.d.periodic[e];
  }
  P.amp = m.d.deform_amp;
  P.left = m.d.deform_left;
  P.right = m.d.deform_right;
  P.freq = m.d.deform_freq;
  return P;
}

GeneralGeom::~GeneralGeom() {
  for (void* p : {(void*)cellG, (void*)face, (void*)ftau, (void*)fnb, (void*)cell_raw, (void*)face_raw, (void*)tau,
                  (void*)bc_dev})
    if (p) cudaFree(p);
}

void GeneralGeom::build(const MeshInfo& m, const FE1D& fe, double ip, int prec, bool keep_raw, cudaStream_t s) {
  precision = prec;
  n_cells = m.n_cells();
  nq = fe.nq;
  long long nq3 = (long long)nq * nq * nq, nq2 = (long long)nq * nq, per = nq3 + 6 * nq2;
  MapParams P = map_params(m, fe);
  EXG_CUDA(cudaMalloc(&cell_raw, n_cells * nq3 * 10 * sizeof(double)));
  EXG_CUDA(cudaMalloc(&face_raw, n_cells * 6 * nq2 * 16 * sizeof(double)));
  EXG_CUDA(cudaMalloc(&tau, n_cells * sizeof(double)));
  EXG_CUDA(cudaMalloc(&bc_dev, 6 * sizeof(int)));
  EXG_CUDA(cudaMemcpyAsync(bc_dev, m.d.bc, 6 * sizeof(int), cudaMemcpyHostToDevice, s));
  long long total = n_cells * per;
  geom_raw_kernel<<<(unsigned)((total + 127) / 128), 128, 0, s>>>(P, n_cells, cell_raw, face_raw);
  EXG_CUDA(cudaGetLastError());
  geom_tau_kernel<<<(unsigned)((n_cells + 127) / 128), 128, 0, s>>>(P, n_cells, cell_raw, face_raw, tau);
  EXG_CUDA(cudaGetLastError());
  size_t ts = prec == EXG_PREC_F32 ? sizeof(float) : sizeof(double);
  EXG_CUDA(cudaMalloc(&cellG, n_cells * nq3 * 6 * ts));
  EXG_CUDA(cudaMalloc(&face, n_cells * 6 * nq2 * 7 * ts));
  EXG_CUDA(cudaMalloc(&ftau, n_cells * 6 * ts));
  EXG_CUDA(cudaMalloc(&fnb, n_cells * 6 * sizeof(long long)));
  double factor = ip * (fe.k + 1.0) * (fe.k + 1.0);
  if (prec == EXG_PREC_F32)
    geom_final_kernel<float><<<(unsigned)((total + 127) / 128), 128, 0, s>>>(
        P, n_cells, factor, bc_dev, cell_raw, face_raw, tau, (float*)cellG, (float*)face, (float*)ftau, fnb);
  else if (prec == EXG_PREC_F64E)
    geom_final_kernel<df64><<<(unsigned)((total + 127) / 128), 128, 0, s>>>(
        P, n_cells, factor, bc_dev, cell_raw, face_raw, tau, (df64*)cellG, (df64*)face, (df64*)ftau, fnb);
  else
    geom_final_kernel<double><<<(unsigned)((total + 127) / 128), 128, 0, s>>>(
        P, n_cells, factor, bc_dev, cell_raw, face_raw, tau, (double*)cellG, (double*)face, (double*)ftau, fnb);
  EXG_CUDA(cudaGetLastError());
  if (!keep_raw) {
    EXG_CUDA(cudaStreamSynchronize(s));
    cudaFree(cell_raw);
    cudaFree(face_raw);
    cell_raw = face_raw = nullptr;
  }
}

// ------------------------------------------------------------------------------------------------
// apply kernel
// ------------------------------------------------------------------------------------------------
template <int N, class C>
struct GenCoef {
  C S[N * N], D[N * N];  // S[q*N + i] = l_i(x_q)
  C d0[N], d1[N];        // l_i'(0), l_i'(1)
};

template <int D, int N>
__device__ __forceinline__ int lidx(int i, int a, int b) {
  return D == 0 ? i + N * (a + N * b) : (D == 1 ? a + N * (i + N * b) : a + N * (b + N * i));
}

// index of the face point (p1, p2) on the face normal to d, at position i along d
__device__ __forceinline__ int fidx(int N, int d, int i, int p1, int p2) {
  return d == 0 ? i + N * (p1 + N * p2) : (d == 1 ? p1 + N * (i + N * p2) : p1 + N * (p2 + N * i));
}

// Per-cell strides of the shared arrays, padded so that the cell strides are congruent to the
// N^2 threads of a cell modulo the 32 banks: consecutive threads of neighbouring cells in one warp
// then address consecutive banks (no conflicts between the cells sharing a warp).
template <int N, class C>
__host__ __device__ constexpr int gen_pad(int len) {
  constexpr int bank = 128 / (int)sizeof(C);
  return len + (((N * N - len) % bank) + bank) % bank;
}
template <int N, class C>
__host__ __device__ constexpr int gen_cell_stride() { return gen_pad<N, C>(N * N * N); }
template <int N, class C>
__host__ __device__ constexpr int gen_face_stride() { return gen_pad<N, C>(28 * N * N); }

// FACES = false: the cell term alone (the continuous levels of cphMG on curved meshes)
template <int N, int CPB, class T, class C, bool FACES = true>
__global__ void __launch_bounds__(CPB* N* N) gen_apply_kernel(const T* __restrict__ src, T* __restrict__ dst,
                                                              const __grid_constant__ GenCoef<N, C> P,
                                                              const C* __restrict__ cellG, const C* __restrict__ face,
                                                              const C* __restrict__ ftau,
                                                              const long long* __restrict__ fnb, long long cell_begin,
                                                              long long n_cells, long long n_dofs,
                                                              const PointEpilogue ep) {
  constexpr int N2 = N * N, N3 = N2 * N, NT = CPB * N2;
  constexpr int SC = gen_cell_stride<N, C>(), SF = gen_face_stride<N, C>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* su = reinterpret_cast<C*>(smem_raw);
  C* so = su + CPB * SC;
  C* t0 = so + CPB * SC;
  C* t1 = t0 + CPB * SC;
  C* t2 = t1 + CPB * SC;
  C* fsh = t2 + CPB * SC;  // CPB * SF face scratch

  // 1D matrices for the face stages, where the row index differs between the threads of a warp:
  // read from shared memory (a kernel-parameter read with a per-thread index is serialised)
  __shared__ C sS[N2], sD[N2];
  for (int i = threadIdx.x; i < N2; i += NT) {
    sS[i] = P.S[i];
    sD[i] = P.D[i];
  }

  const long long c0 = cell_begin + (long long)blockIdx.x * CPB;  // cells [cell_begin, n_cells)
  const T* s = src + (long long)blockIdx.y * n_dofs;
  T* o = dst + (long long)blockIdx.y * n_dofs;
  const int tid = threadIdx.x;
  const long long base = c0 * N3;
  const long long nch = min((long long)CPB, n_cells - c0);
  const int nd = (int)(nch * N3);
  for (int i = tid; i < CPB * N3; i += NT) {
    const int lcc = i / N3, e = lcc * SC + i - lcc * N3;
    su[e] = i < nd ? load_as<C>(s + base + i) : C(0);
    so[e] = C(0);
  }
  __syncthreads();
  const int lc = tid / N2, l = tid - lc * N2, a = l % N, b = l / N;
  const bool active = lc < nch;
  const long long c = c0 + lc;
  const int co = lc * SC;
  C* U = su + co;
  C* A0 = t0 + co;
  C* A1 = t1 + co;
  C* A2 = t2 + co;
  // ---- cell term: gradients at q (x, then y, then z), G, transpose back
  if (active) {  // x-lines (j=a, k=b)
    C u[N];
#pragma unroll
    for (int i = 0; i < N; ++i) u[i] = U[lidx<0, N>(i, a, b)];
#pragma unroll
    for (int q = 0; q < N; ++q) {
      C vs = C(0), vd = C(0);
#pragma unroll
      for (int i = 0; i < N; ++i) {
        vs = fmadd(P.S[q * N + i], u[i], vs);
        vd = fmadd(P.D[q * N + i], u[i], vd);
      }
      A0[lidx<0, N>(q, a, b)] = vs;  // A = S_x u
      A1[lidx<0, N>(q, a, b)] = vd;  // B = D_x u
    }
  }
  __syncthreads();
  if (active) {  // y-lines (i=a, k=b): C = S_y A, E = D_y A, F = S_y B
    C va[N], vb[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      va[i] = A0[lidx<1, N>(i, a, b)];
      vb[i] = A1[lidx<1, N>(i, a, b)];
    }
#pragma unroll
    for (int q = 0; q < N; ++q) {
      C cs = C(0), ce = C(0), cf = 0;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        cs = fmadd(P.S[q * N + i], va[i], cs);
        ce = fmadd(P.D[q * N + i], va[i], ce);
        cf = fmadd(P.S[q * N + i], vb[i], cf);
      }
      A0[lidx<1, N>(q, a, b)] = cs;
      A1[lidx<1, N>(q, a, b)] = ce;
      A2[lidx<1, N>(q, a, b)] = cf;
    }
  }
  __syncthreads();
  if (active) {  // z-lines (i=a, j=b): g2 = D_z C, g1 = S_z E, g0 = S_z F; flux; transpose
    C vc[N], ve[N], vf[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      vc[i] = A0[lidx<2, N>(i, a, b)];
      ve[i] = A1[lidx<2, N>(i, a, b)];
      vf[i] = A2[lidx<2, N>(i, a, b)];
    }
    C f0[N], f1[N], f2[N];
#pragma unroll
    for (int q = 0; q < N; ++q) {
      C g0 = C(0), g1 = C(0), g2 = 0;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        g0 = fmadd(P.S[q * N + i], vf[i], g0);
        g1 = fmadd(P.S[q * N + i], ve[i], g1);
        g2 = fmadd(P.D[q * N + i], vc[i], g2);
      }
      const C* G = cellG + (c * N3 + lidx<2, N>(q, a, b)) * 6;
      C G00 = G[0], G01 = G[1], G02 = G[2], G11 = G[3], G12 = G[4], G22 = G[5];
      f0[q] = G00 * g0 + G01 * g1 + G02 * g2;
      f1[q] = G01 * g0 + G11 * g1 + G12 * g2;
      f2[q] = G02 * g0 + G12 * g1 + G22 * g2;
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
      C xf = C(0), xe = C(0), xc = 0;
#pragma unroll
      for (int q = 0; q < N; ++q) {
        xf = fmadd(P.S[q * N + i], f0[q], xf);
        xe = fmadd(P.S[q * N + i], f1[q], xe);
        xc = fmadd(P.D[q * N + i], f2[q], xc);
      }
      A2[lidx<2, N>(i, a, b)] = xf;  // F'
      A1[lidx<2, N>(i, a, b)] = xe;  // E'
      A0[lidx<2, N>(i, a, b)] = xc;  // C'
    }
  }
  __syncthreads();
  if (active) {  // y-lines: A' = S^T C' + D^T E', B' = S^T F'
    C vc[N], ve[N], vf[N];
#pragma unroll
    for (int q = 0; q < N; ++q) {
      vc[q] = A0[lidx<1, N>(q, a, b)];
      ve[q] = A1[lidx<1, N>(q, a, b)];
      vf[q] = A2[lidx<1, N>(q, a, b)];
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
      C xa = C(0), xb = C(0);
#pragma unroll
      for (int q = 0; q < N; ++q) {
        xa = fmadd(P.S[q * N + i], vc[q], xa);
        xa = fmadd(P.D[q * N + i], ve[q], xa);
        xb = fmadd(P.S[q * N + i], vf[q], xb);
      }
      A0[lidx<1, N>(i, a, b)] = xa;
      A1[lidx<1, N>(i, a, b)] = xb;
    }
  }
  __syncthreads();
  if (active) {  // x-lines: out = S^T A' + D^T B'
    C va[N], vb[N];
#pragma unroll
    for (int q = 0; q < N; ++q) {
      va[q] = A0[lidx<0, N>(q, a, b)];
      vb[q] = A1[lidx<0, N>(q, a, b)];
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
      C x = C(0);
#pragma unroll
      for (int q = 0; q < N; ++q) {
        x = fmadd(P.S[q * N + i], va[q], x);
        x = fmadd(P.D[q * N + i], vb[q], x);
      }
      so[co + lidx<0, N>(i, a, b)] = x;
    }
  }
  __syncthreads();
  // ---- face terms, both faces of a direction per pass (independent work for the two faces in
  // every stage, half the barriers).  Per face: traces (A), interpolation along t1 (1) and t2 plus
  // the flux (2), transposed interpolation along t2 (E) and t1 with accumulation into the lines
  // along d (F).  Each face has its own 14 N^2 scratch arrays.
  C* F = fsh + lc * SF;
  const int p1 = a, p2 = b;  // this thread's face point / node
#pragma unroll 1
  for (int d = 0; d < (FACES ? 3 : 0); ++d) {
    int t1d, t2d;
    tang(d, t1d, t2d);
    const long long nbs[2] = {active ? fnb[c * 6 + 2 * d] : -2, active ? fnb[c * 6 + 2 * d + 1] : -2};
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const int f = 2 * d + side;
      const long long nb = nbs[side];
      const bool interior = nb >= 0;
      const C* dside = side ? P.d1 : P.d0;
      const C* dopp = side ? P.d0 : P.d1;
      const int iend = side ? N - 1 : 0, iopp = side ? 0 : N - 1;
      C* Fs = F + side * 14 * N2;
      C* fv = Fs;
      C* fn = Fs + N2;
      C* gv = Fs + 2 * N2;
      C* gn = Fs + 3 * N2;
      C* r0 = Fs + 4 * N2;
      C* r1 = Fs + 5 * N2;
      C* r2 = Fs + 6 * N2;
      C* r3 = Fs + 7 * N2;
      C* r4 = Fs + 8 * N2;
      C* r5 = Fs + 9 * N2;
      C* cv = Fs + 10 * N2;
      C* c0_ = Fs + 11 * N2;
      C* c1_ = Fs + 12 * N2;
      C* c2_ = Fs + 13 * N2;
      (void)f, (void)interior, (void)dside, (void)dopp, (void)iend, (void)iopp, (void)fv, (void)fn, (void)gv,
          (void)gn, (void)r0, (void)r1, (void)r2, (void)r3, (void)r4, (void)r5, (void)cv, (void)c0_, (void)c1_,
          (void)c2_;
      if (active) {
        C nd = C(0);
        for (int i = 0; i < N; ++i) nd = fmadd(dside[i], U[fidx(N, d, i, p1, p2)], nd);
        fv[p2 * N + p1] = U[fidx(N, d, iend, p1, p2)];
        fn[p2 * N + p1] = nd;
        if (interior) {
          const T* un = s + nb * N3;
          C ndn = C(0);
          for (int i = 0; i < N; ++i) ndn = fmadd(dopp[i], load_as<C>(un + fidx(N, d, i, p1, p2)), ndn);
          gv[p2 * N + p1] = load_as<C>(un + fidx(N, d, iopp, p1, p2));
          gn[p2 * N + p1] = ndn;
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const int f = 2 * d + side;
      const long long nb = nbs[side];
      const bool interior = nb >= 0;
      const C* dside = side ? P.d1 : P.d0;
      const C* dopp = side ? P.d0 : P.d1;
      const int iend = side ? N - 1 : 0, iopp = side ? 0 : N - 1;
      C* Fs = F + side * 14 * N2;
      C* fv = Fs;
      C* fn = Fs + N2;
      C* gv = Fs + 2 * N2;
      C* gn = Fs + 3 * N2;
      C* r0 = Fs + 4 * N2;
      C* r1 = Fs + 5 * N2;
      C* r2 = Fs + 6 * N2;
      C* r3 = Fs + 7 * N2;
      C* r4 = Fs + 8 * N2;
      C* r5 = Fs + 9 * N2;
      C* cv = Fs + 10 * N2;
      C* c0_ = Fs + 11 * N2;
      C* c1_ = Fs + 12 * N2;
      C* c2_ = Fs + 13 * N2;
      (void)f, (void)interior, (void)dside, (void)dopp, (void)iend, (void)iopp, (void)fv, (void)fn, (void)gv,
          (void)gn, (void)r0, (void)r1, (void)r2, (void)r3, (void)r4, (void)r5, (void)cv, (void)c0_, (void)c1_,
          (void)c2_;
      if (active && nb != -2) {
        C sv = C(0), sdv = C(0), sn = 0, nv = C(0), ndv = 0, nn = C(0);
        for (int k = 0; k < N; ++k) {
          C Sq = sS[p1 * N + k], Dq = sD[p1 * N + k];
          sv = fmadd(Sq, fv[p2 * N + k], sv);
          sdv = fmadd(Dq, fv[p2 * N + k], sdv);
          sn = fmadd(Sq, fn[p2 * N + k], sn);
          if (interior) {
            nv = fmadd(Sq, gv[p2 * N + k], nv);
            ndv = fmadd(Dq, gv[p2 * N + k], ndv);
            nn = fmadd(Sq, gn[p2 * N + k], nn);
          }
        }
        r0[p2 * N + p1] = sv;
        r1[p2 * N + p1] = sdv;
        r2[p2 * N + p1] = sn;
        r3[p2 * N + p1] = nv;
        r4[p2 * N + p1] = ndv;
        r5[p2 * N + p1] = nn;
      }
    }
    __syncthreads();
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const int f = 2 * d + side;
      const long long nb = nbs[side];
      const bool interior = nb >= 0;
      const C* dside = side ? P.d1 : P.d0;
      const C* dopp = side ? P.d0 : P.d1;
      const int iend = side ? N - 1 : 0, iopp = side ? 0 : N - 1;
      C* Fs = F + side * 14 * N2;
      C* fv = Fs;
      C* fn = Fs + N2;
      C* gv = Fs + 2 * N2;
      C* gn = Fs + 3 * N2;
      C* r0 = Fs + 4 * N2;
      C* r1 = Fs + 5 * N2;
      C* r2 = Fs + 6 * N2;
      C* r3 = Fs + 7 * N2;
      C* r4 = Fs + 8 * N2;
      C* r5 = Fs + 9 * N2;
      C* cv = Fs + 10 * N2;
      C* c0_ = Fs + 11 * N2;
      C* c1_ = Fs + 12 * N2;
      C* c2_ = Fs + 13 * N2;
      (void)f, (void)interior, (void)dside, (void)dopp, (void)iend, (void)iopp, (void)fv, (void)fn, (void)gv,
          (void)gn, (void)r0, (void)r1, (void)r2, (void)r3, (void)r4, (void)r5, (void)cv, (void)c0_, (void)c1_,
          (void)c2_;
      if (active && nb != -2) {
        C vo = C(0), go_t1 = C(0), go_t2 = 0, go_d = C(0), vn = 0, gn_t1 = C(0), gn_t2 = 0, gn_d = C(0);
        for (int k = 0; k < N; ++k) {
          C Sq = sS[p2 * N + k], Dq = sD[p2 * N + k];
          vo = fmadd(Sq, r0[k * N + p1], vo);
          go_t2 = fmadd(Dq, r0[k * N + p1], go_t2);
          go_t1 = fmadd(Sq, r1[k * N + p1], go_t1);
          go_d = fmadd(Sq, r2[k * N + p1], go_d);
          if (interior) {
            vn = fmadd(Sq, r3[k * N + p1], vn);
            gn_t2 = fmadd(Dq, r3[k * N + p1], gn_t2);
            gn_t1 = fmadd(Sq, r4[k * N + p1], gn_t1);
            gn_d = fmadd(Sq, r5[k * N + p1], gn_d);
          }
        }
        const C* fd = face + ((c * 6 + f) * N2 + p2 * N + p1) * 7;
        C ao[3] = {fd[0], fd[1], fd[2]};
        C JxW = fd[6];
        // reference gradient components by direction, through selects (a runtime index into a small
        // array would put it in local memory)
        const C go0 = d == 0 ? go_d : (t1d == 0 ? go_t1 : go_t2);
        const C go1 = d == 1 ? go_d : (t1d == 1 ? go_t1 : go_t2);
        const C go2 = d == 2 ? go_d : (t1d == 2 ? go_t1 : go_t2);
        C ndo = ao[0] * go0 + ao[1] * go1 + ao[2] * go2;
        C tau = ftau[c * 6 + f];
        C gflux, sv;
        if (interior) {
          C an[3] = {fd[3], fd[4], fd[5]};
          const C gn0 = d == 0 ? gn_d : (t1d == 0 ? gn_t1 : gn_t2);
          const C gn1 = d == 1 ? gn_d : (t1d == 1 ? gn_t1 : gn_t2);
          const C gn2 = d == 2 ? gn_d : (t1d == 2 ? gn_t1 : gn_t2);
          C ndn = an[0] * gn0 + an[1] * gn1 + an[2] * gn2;
          const bool own_minus = side == 1;
          C um = own_minus ? vo : vn, up = own_minus ? vn : vo;
          C nm = own_minus ? ndo : ndn, np = own_minus ? ndn : ndo;
          gflux = cconst<C>(-0.5) * (um - up);
          C vflux = cconst<C>(0.5) * (nm + np) - tau * (um - up);
          sv = own_minus ? neg(vflux) : vflux;
        } else {  // homogeneous Dirichlet: u+ = -u-, du+/dn = du-/dn
          gflux = neg(vo);
          sv = neg(ndo - cconst<C>(2.0) * tau * vo);
        }
        cv[p2 * N + p1] = JxW * sv;
        C gj = JxW * gflux;
        const C a_d = d == 0 ? ao[0] : (d == 1 ? ao[1] : ao[2]);
        const C a_t1 = t1d == 0 ? ao[0] : (t1d == 1 ? ao[1] : ao[2]);
        const C a_t2 = t2d == 0 ? ao[0] : (t2d == 1 ? ao[1] : ao[2]);
        c0_[p2 * N + p1] = gj * a_d;
        c1_[p2 * N + p1] = gj * a_t1;
        c2_[p2 * N + p1] = gj * a_t2;
      }
    }
    __syncthreads();
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const int f = 2 * d + side;
      const long long nb = nbs[side];
      const bool interior = nb >= 0;
      const C* dside = side ? P.d1 : P.d0;
      const C* dopp = side ? P.d0 : P.d1;
      const int iend = side ? N - 1 : 0, iopp = side ? 0 : N - 1;
      C* Fs = F + side * 14 * N2;
      C* fv = Fs;
      C* fn = Fs + N2;
      C* gv = Fs + 2 * N2;
      C* gn = Fs + 3 * N2;
      C* r0 = Fs + 4 * N2;
      C* r1 = Fs + 5 * N2;
      C* r2 = Fs + 6 * N2;
      C* r3 = Fs + 7 * N2;
      C* r4 = Fs + 8 * N2;
      C* r5 = Fs + 9 * N2;
      C* cv = Fs + 10 * N2;
      C* c0_ = Fs + 11 * N2;
      C* c1_ = Fs + 12 * N2;
      C* c2_ = Fs + 13 * N2;
      (void)f, (void)interior, (void)dside, (void)dopp, (void)iend, (void)iopp, (void)fv, (void)fn, (void)gv,
          (void)gn, (void)r0, (void)r1, (void)r2, (void)r3, (void)r4, (void)r5, (void)cv, (void)c0_, (void)c1_,
          (void)c2_;
      if (active && nb != -2) {
        C s1 = C(0), s2 = C(0), s3 = 0, s4 = C(0);
        for (int q = 0; q < N; ++q) {
          C Sq = sS[q * N + p2], Dq = sD[q * N + p2];
          s1 = fmadd(Sq, cv[q * N + p1], s1);
          s2 = fmadd(Sq, c1_[q * N + p1], s2);
          s3 = fmadd(Dq, c2_[q * N + p1], s3);
          s4 = fmadd(Sq, c0_[q * N + p1], s4);
        }
        r0[p2 * N + p1] = s1;
        r1[p2 * N + p1] = s2;
        r2[p2 * N + p1] = s3;
        r3[p2 * N + p1] = s4;
      }
    }
    __syncthreads();
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const int f = 2 * d + side;
      const long long nb = nbs[side];
      const bool interior = nb >= 0;
      const C* dside = side ? P.d1 : P.d0;
      const C* dopp = side ? P.d0 : P.d1;
      const int iend = side ? N - 1 : 0, iopp = side ? 0 : N - 1;
      C* Fs = F + side * 14 * N2;
      C* fv = Fs;
      C* fn = Fs + N2;
      C* gv = Fs + 2 * N2;
      C* gn = Fs + 3 * N2;
      C* r0 = Fs + 4 * N2;
      C* r1 = Fs + 5 * N2;
      C* r2 = Fs + 6 * N2;
      C* r3 = Fs + 7 * N2;
      C* r4 = Fs + 8 * N2;
      C* r5 = Fs + 9 * N2;
      C* cv = Fs + 10 * N2;
      C* c0_ = Fs + 11 * N2;
      C* c1_ = Fs + 12 * N2;
      C* c2_ = Fs + 13 * N2;
      (void)f, (void)interior, (void)dside, (void)dopp, (void)iend, (void)iopp, (void)fv, (void)fn, (void)gv,
          (void)gn, (void)r0, (void)r1, (void)r2, (void)r3, (void)r4, (void)r5, (void)cv, (void)c0_, (void)c1_,
          (void)c2_;
      if (active && nb != -2) {
        C tv = C(0), tn = C(0);
        for (int q = 0; q < N; ++q) {
          C Sq = sS[q * N + p1], Dq = sD[q * N + p1];
          tv = fmadd(Sq, r0[p2 * N + q], tv);
          tv = fmadd(Dq, r1[p2 * N + q], tv);
          tv = fmadd(Sq, r2[p2 * N + q], tv);
          tn = fmadd(Sq, r3[p2 * N + q], tn);
        }
        so[co + fidx(N, d, iend, p1, p2)] = so[co + fidx(N, d, iend, p1, p2)] + tv;
        for (int i = 0; i < N; ++i) so[co + fidx(N, d, i, p1, p2)] = fmadd(dside[i], tn, so[co + fidx(N, d, i, p1, p2)]);
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < nd; i += NT) {
    const int lcc = i / N3;
    epilogue_store<T>(ep, o, base + i, s, to_storage<T>(so[lcc * SC + i - lcc * N3]));
  }
}

template <int N, class C>
static GenCoef<N, C> gen_coef(const FE1D& fe) {
  GenCoef<N, C> P;
  for (int i = 0; i < N * N; ++i) {
    P.S[i] = coef_from_double<C>(fe.S[i]);
    P.D[i] = coef_from_double<C>(fe.D[i]);
  }
  for (int i = 0; i < N; ++i) {
    P.d0[i] = coef_from_double<C>(fe.dL[i]);
    P.d1[i] = coef_from_double<C>(fe.dR[i]);
  }
  return P;
}

template <int N>
constexpr int gen_cpb() {
  return N <= 3 ? 16 : (N <= 5 ? 8 : (N <= 7 ? 4 : 2));
}

template <int N, class T, class C>
static void gen_apply_n(const GeneralGeom& g, const FE1D& fe, const void* src, void* dst, int n_rhs, cudaStream_t s,
                        const PointEpilogue& ep, long long cb, long long ce) {
  constexpr int CPB = gen_cpb<N>(), N3 = N * N * N, N2 = N * N;
  GenCoef<N, C> P = gen_coef<N, C>(fe);
  const bool faces = !g.cell_only;
  size_t smem = (5 * (size_t)CPB * gen_cell_stride<N, C>() + (faces ? (size_t)CPB * gen_face_stride<N, C>() : 0)) *
                sizeof(C);
  auto kern = faces ? gen_apply_kernel<N, CPB, T, C, true> : gen_apply_kernel<N, CPB, T, C, false>;
  ensure_smem_attr((const void*)kern, (int)smem);
  long long blocks = (ce - cb + CPB - 1) / CPB;
  dim3 grid((unsigned)blocks, (unsigned)n_rhs);
  kern<<<grid, CPB * N2, smem, s>>>((const T*)src, (T*)dst, P, (const C*)g.cellG, (const C*)g.face, (const C*)g.ftau,
                                    g.fnb, cb, ce, g.n_cells * N3, ep);
  EXG_CUDA(cudaGetLastError());
}

template <class T, class C>
static void gen_apply_t(const GeneralGeom& g, const FE1D& fe, const void* src, void* dst, int n_rhs, cudaStream_t s,
                        const PointEpilogue& ep, long long cb, long long ce) {
  switch (fe.n) {
    case 2: gen_apply_n<2, T, C>(g, fe, src, dst, n_rhs, s, ep, cb, ce); break;
    case 3: gen_apply_n<3, T, C>(g, fe, src, dst, n_rhs, s, ep, cb, ce); break;
    case 4: gen_apply_n<4, T, C>(g, fe, src, dst, n_rhs, s, ep, cb, ce); break;
    case 5: gen_apply_n<5, T, C>(g, fe, src, dst, n_rhs, s, ep, cb, ce); break;
    case 6: gen_apply_n<6, T, C>(g, fe, src, dst, n_rhs, s, ep, cb, ce); break;
    case 7: gen_apply_n<7, T, C>(g, fe, src, dst, n_rhs, s, ep, cb, ce); break;
    case 8: gen_apply_n<8, T, C>(g, fe, src, dst, n_rhs, s, ep, cb, ce); break;
    case 9: gen_apply_n<9, T, C>(g, fe, src, dst, n_rhs, s, ep, cb, ce); break;
    default: throw Error{EXG_ERR_UNSUPPORTED, "degree must be 1..8"};
  }
}

void general_apply(const GeneralGeom& g, const FE1D& fe, const void* src, void* dst, int n_rhs, cudaStream_t s,
                   const PointEpilogue& ep, long long cell_begin, long long cell_end) {
  if (cell_end < 0) cell_end = g.n_cells;
  EXG_CHECK(cell_begin >= 0 && cell_begin < cell_end && cell_end <= g.n_cells, EXG_ERR_INVALID, "bad cell range");
  EXG_CHECK(n_rhs >= 1 && n_rhs <= 65535, EXG_ERR_INVALID, "n_rhs out of range");
  EXG_CHECK(ep.mode < 0 || n_rhs == 1, EXG_ERR_INVALID, "fused point update needs a single right-hand side");
  if (g.precision == EXG_PREC_F32)
    gen_apply_t<float, float>(g, fe, src, dst, n_rhs, s, ep, cell_begin, cell_end);
  else if (g.precision == EXG_PREC_F64E)
    gen_apply_t<double, df64>(g, fe, src, dst, n_rhs, s, ep, cell_begin, cell_end);
  else
    gen_apply_t<double, double>(g, fe, src, dst, n_rhs, s, ep, cell_begin, cell_end);
}

// ------------------------------------------------------------------------------------------------
// diagonal (thread per DoF), rhs (thread per DoF), quadrature points
// ------------------------------------------------------------------------------------------------
struct FETab {
  int n;
  double S[100], D[100], d0[10], d1[10];
};

template <class TG, class TO>
__global__ void gen_diag_kernel(FETab F, const TG* __restrict__ cellG, const TG* __restrict__ face,
                                const TG* __restrict__ ftau, const long long* __restrict__ fnb, long long n_dofs,
                                TO* __restrict__ out, bool invert) {
  const int n = F.n, n2 = n * n, n3 = n2 * n;
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_dofs) return;
  long long c = g / n3;
  int loc = (int)(g - c * n3);
  int ix[3] = {loc % n, (loc / n) % n, loc / n2};
  double sum = 0;
  for (int q2 = 0; q2 < n; ++q2)
    for (int q1 = 0; q1 < n; ++q1)
      for (int q0 = 0; q0 < n; ++q0) {
        int qs[3] = {q0, q1, q2};
        double gr[3];
        for (int k = 0; k < 3; ++k) {
          double v = 1;
          for (int e = 0; e < 3; ++e) v *= (e == k ? F.D : F.S)[qs[e] * n + ix[e]];
          gr[k] = v;
        }
        const TG* G = cellG + (c * n3 + (q2 * n + q1) * n + q0) * 6;
        double G00 = coef_to_double(G[0]), G01 = coef_to_double(G[1]), G02 = coef_to_double(G[2]),
               G11 = coef_to_double(G[3]), G12 = coef_to_double(G[4]), G22 = coef_to_double(G[5]);
        sum += gr[0] * (G00 * gr[0] + G01 * gr[1] + G02 * gr[2]) + gr[1] * (G01 * gr[0] + G11 * gr[1] + G12 * gr[2]) +
               gr[2] * (G02 * gr[0] + G12 * gr[1] + G22 * gr[2]);
      }
  for (int f = 0; f < 6; ++f) {
    int d = f / 2, side = f % 2, t1, t2;
    tang(d, t1, t2);
    int iend = side ? n - 1 : 0;
    if (ix[d] != iend) continue;  // GL basis: only face nodes have a trace on the face
    long long nb = fnb[c * 6 + f];
    if (nb == -2) continue;  // Neumann
    double tau = coef_to_double(ftau[c * 6 + f]);
    const double* dside = side ? F.d1 : F.d0;
    for (int q2 = 0; q2 < n; ++q2)
      for (int q1 = 0; q1 < n; ++q1) {
        const TG* fd = face + ((c * 6 + f) * n2 + q2 * n + q1) * 7;
        double v = F.S[q1 * n + ix[t1]] * F.S[q2 * n + ix[t2]];
        double gr[3];
        gr[d] = dside[ix[d]] * F.S[q1 * n + ix[t1]] * F.S[q2 * n + ix[t2]];
        gr[t1] = F.D[q1 * n + ix[t1]] * F.S[q2 * n + ix[t2]];
        gr[t2] = F.S[q1 * n + ix[t1]] * F.D[q2 * n + ix[t2]];
        double nd = coef_to_double(fd[0]) * gr[0] + coef_to_double(fd[1]) * gr[1] + coef_to_double(fd[2]) * gr[2];
        double JxW = coef_to_double(fd[6]);
        if (nb >= 0) {
          double s = side == 1 ? -1.0 : 1.0;
          sum += JxW * (s * v * nd + tau * v * v);
        } else {
          sum += JxW * (-2.0 * v * nd + 2.0 * tau * v * v);
        }
      }
  }
  TO r = (TO)sum;
  if (invert) r = fabs((double)r) > 1e-10 ? (TO)1 / r : (TO)1;
  out[g] = r;
}

// b_i = (f, phi_i) - inhomogeneous boundary part, FP64
__global__ void gen_rhs_kernel(FETab F, const double* __restrict__ cell_raw, const double* __restrict__ face,
                               const double* __restrict__ ftau, const long long* __restrict__ fnb,
                               const double* __restrict__ fq, const double* __restrict__ gq,
                               const double* __restrict__ hq, long long n_dofs, double* __restrict__ b) {
  const int n = F.n, n2 = n * n, n3 = n2 * n;
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_dofs) return;
  long long c = g / n3;
  int loc = (int)(g - c * n3);
  int ix[3] = {loc % n, (loc / n) % n, loc / n2};
  double sum = 0;
  if (fq)
    for (int q2 = 0; q2 < n; ++q2)
      for (int q1 = 0; q1 < n; ++q1)
        for (int q0 = 0; q0 < n; ++q0) {
          long long qi = c * n3 + (q2 * n + q1) * n + q0;
          double phi = F.S[q0 * n + ix[0]] * F.S[q1 * n + ix[1]] * F.S[q2 * n + ix[2]];
          sum += fq[qi] * cell_raw[qi * 10 + 6] * phi;
        }
  for (int f = 0; f < 6; ++f) {
    long long nb = fnb[c * 6 + f];
    if (nb >= 0) continue;
    int d = f / 2, side = f % 2, t1, t2;
    tang(d, t1, t2);
    const double* dside = side ? F.d1 : F.d0;
    int iend = side ? n - 1 : 0;
    double tau = ftau[c * 6 + f];
    for (int q2 = 0; q2 < n; ++q2)
      for (int q1 = 0; q1 < n; ++q1) {
        long long fi = (c * 6 + f) * n2 + q2 * n + q1;
        const double* fd = face + fi * 7;
        double v = ix[d] == iend ? F.S[q1 * n + ix[t1]] * F.S[q2 * n + ix[t2]] : 0.0;
        double gr[3];
        gr[d] = dside[ix[d]] * F.S[q1 * n + ix[t1]] * F.S[q2 * n + ix[t2]];
        gr[t1] = ix[d] == iend ? F.D[q1 * n + ix[t1]] * F.S[q2 * n + ix[t2]] : 0.0;
        gr[t2] = ix[d] == iend ? F.S[q1 * n + ix[t1]] * F.D[q2 * n + ix[t2]] : 0.0;
        double nd = fd[0] * gr[0] + fd[1] * gr[1] + fd[2] * gr[2];
        double JxW = fd[6];
        if (nb == -1) {
          // Dirichlet: phi- = 0, phi+ = 2g: gflux = g, vflux = 2 tau g; rhs -= (g nd - 2 tau g v)
          double gv = gq ? gq[fi] : 0.0;
          sum -= JxW * (gv * nd - 2.0 * tau * gv * v);
        } else {
          // Neumann: vflux = h; rhs -= (-h v)
          double hv = hq ? hq[fi] : 0.0;
          sum += JxW * hv * v;
        }
      }
  }
  b[g] = sum;
}

__global__ void gen_points_kernel(const double* __restrict__ cell_raw, const double* __restrict__ face_raw,
                                  long long n_cell_pts, long long n_face_pts, double* __restrict__ cx,
                                  double* __restrict__ fx) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n_cell_pts) {
    if (cx)
      for (int e = 0; e < 3; ++e) cx[g * 3 + e] = cell_raw[g * 10 + 7 + e];
  } else if (g < n_cell_pts + n_face_pts) {
    long long h = g - n_cell_pts;
    if (fx)
      for (int e = 0; e < 3; ++e) fx[h * 3 + e] = face_raw[h * 16 + 13 + e];
  }
}

static FETab fetab(const FE1D& fe) {
  FETab F{};
  F.n = fe.n;
  for (int i = 0; i < fe.n * fe.n; ++i) {
    F.S[i] = fe.S[i];
    F.D[i] = fe.D[i];
  }
  for (int i = 0; i < fe.n; ++i) {
    F.d0[i] = fe.dL[i];
    F.d1[i] = fe.dR[i];
  }
  return F;
}

void general_diagonal(const GeneralGeom& g, const FE1D& fe, void* out, bool invert, cudaStream_t s) {
  long long nd = g.n_cells * fe.n * fe.n * fe.n;
  FETab F = fetab(fe);
  if (g.precision == EXG_PREC_F32)
    gen_diag_kernel<float, float><<<(unsigned)((nd + 127) / 128), 128, 0, s>>>(
        F, (const float*)g.cellG, (const float*)g.face, (const float*)g.ftau, g.fnb, nd, (float*)out, invert);
  else if (g.precision == EXG_PREC_F64E)
    gen_diag_kernel<df64, double><<<(unsigned)((nd + 127) / 128), 128, 0, s>>>(
        F, (const df64*)g.cellG, (const df64*)g.face, (const df64*)g.ftau, g.fnb, nd, (double*)out, invert);
  else
    gen_diag_kernel<double, double><<<(unsigned)((nd + 127) / 128), 128, 0, s>>>(
        F, (const double*)g.cellG, (const double*)g.face, (const double*)g.ftau, g.fnb, nd, (double*)out, invert);
  EXG_CUDA(cudaGetLastError());
}

void general_rhs(const GeneralGeom& g, const FE1D& fe, const double* fq, const double* gq, const double* hq, double* b,
                 cudaStream_t s) {
  EXG_CHECK(g.precision != EXG_PREC_F32 && g.cell_raw, EXG_ERR_INVALID, "rhs needs FP64 geometry with raw data");
  long long nd = g.n_cells * fe.n * fe.n * fe.n;
  FETab F = fetab(fe);
  gen_rhs_kernel<<<(unsigned)((nd + 127) / 128), 128, 0, s>>>(F, g.cell_raw, (const double*)g.face,
                                                              (const double*)g.ftau, g.fnb, fq, gq, hq, nd, b);
  EXG_CUDA(cudaGetLastError());
}

void general_points(const GeneralGeom& g, double* cx, double* fx, long long* ncp, long long* nfp, cudaStream_t s) {
  long long nq = g.nq;
  long long n_cell_pts = g.n_cells * nq * nq * nq, n_face_pts = g.n_cells * 6 * nq * nq;
  if (ncp) *ncp = n_cell_pts;
  if (nfp) *nfp = n_face_pts;
  if (!cx && !fx) return;
  EXG_CHECK(g.cell_raw, EXG_ERR_INVALID, "geometry built without raw data");
  long long tot = n_cell_pts + n_face_pts;
  gen_points_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(g.cell_raw, g.face_raw, n_cell_pts, n_face_pts, cx,
                                                                  fx);
  EXG_CUDA(cudaGetLastError());
}

}  // namespace exg
