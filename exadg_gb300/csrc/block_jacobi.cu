// Block Jacobi for the SIPG operator on Cartesian meshes: dst = blockdiag(A)^-1 src, the inverse
// of every cell's diagonal block (OperatorBase::apply_inverse_block_diagonal,
// operators/operator_base.cpp:820-900; used as the Krylov preconditioner BlockJacobi).
//
// On a box cell the diagonal block is a Kronecker sum: A_cc = T_x (x) M_y (x) M_z + M_x (x) T_y (x) M_z
// + M_x (x) M_y (x) T_z, with M_d = h_d M_ref the 1D mass matrix and T_d the 1D stiffness K_ref / h_d
// plus the cell's own side of its two faces normal to d (laplace_operator.cpp:139-163, 221-265 with
// the neighbour's values zero: interior and periodic faces -1/2 (d_n u v + u d_n v) + tau' u v with
// tau' = max(tau-, tau+) (k+1)^2 IP; Dirichlet faces twice that with tau_c; Neumann faces nothing).
// The face integrals of tangential products are exactly M_e (x) M_f with k+1 Gauss points.
// Fast diagonalisation: T_d S_d = M_d S_d diag(lambda_d), S_d^T M_d S_d = I, so
//   A_cc^-1 = (S_x (x) S_y (x) S_z) diag(1 / (lambda_x + lambda_y + lambda_z)) (S_x (x) S_y (x) S_z)^T,
// exact up to rounding.  The 1D problem depends on a cell's face kinds and penalties along d only,
// so a few classes per direction cover the mesh (host set-up); the kernel applies the two
// sum-factorised sweeps with the cell's three classes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <tuple>

#include "block_jacobi.h"

namespace exg {

BlockJacobi::~BlockJacobi() {
  for (void* p : {(void*)cls, S, lam})
    if (p) cudaFree(p);
}

// generalised symmetric eigenproblem T S = M S diag(lam), S^T M S = I (Cholesky of M, cyclic
// Jacobi rotations on L^-1 T L^-T); n <= 9
static void gen_eig(int n, const std::vector<double>& T, const std::vector<double>& M, std::vector<double>& S,
                    std::vector<double>& lam) {
  std::vector<double> L(n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = M[i * n + j];
      for (int k = 0; k < j; ++k) s -= L[i * n + k] * L[j * n + k];
      if (i == j) {
        EXG_CHECK(s > 0, EXG_ERR_INVALID, "mass matrix not positive definite");
        L[i * n + i] = std::sqrt(s);
      } else {
        L[i * n + j] = s / L[j * n + j];
      }
    }
  // X = L^-1 T, then C = X L^-T (forward substitutions)
  std::vector<double> X(n * n), C(n * n);
  for (int c = 0; c < n; ++c)
    for (int i = 0; i < n; ++i) {
      double s = T[i * n + c];
      for (int k = 0; k < i; ++k) s -= L[i * n + k] * X[k * n + c];
      X[i * n + c] = s / L[i * n + i];
    }
  for (int r = 0; r < n; ++r)
    for (int j = 0; j < n; ++j) {
      double s = X[r * n + j];
      for (int k = 0; k < j; ++k) s -= C[r * n + k] * L[j * n + k];
      C[r * n + j] = s / L[j * n + j];
    }
  for (int i = 0; i < n; ++i)  // symmetrise the rounding
    for (int j = 0; j < i; ++j) C[i * n + j] = C[j * n + i] = 0.5 * (C[i * n + j] + C[j * n + i]);
  std::vector<double> Q(n * n, 0.0);
  for (int i = 0; i < n; ++i) Q[i * n + i] = 1.0;
  double scale = 0;
  for (int i = 0; i < n * n; ++i) scale += C[i] * C[i];
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += C[p * n + q] * C[p * n + q];
    if (off <= 1e-34 * scale) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = C[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (C[q * n + q] - C[p * n + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // C <- J^T C J
          const double ckp = C[k * n + p], ckq = C[k * n + q];
          C[k * n + p] = c * ckp - s * ckq;
          C[k * n + q] = s * ckp + c * ckq;
        }
        for (int k = 0; k < n; ++k) {
          const double cpk = C[p * n + k], cqk = C[q * n + k];
          C[p * n + k] = c * cpk - s * cqk;
          C[q * n + k] = s * cpk + c * cqk;
        }
        for (int k = 0; k < n; ++k) {
          const double qkp = Q[k * n + p], qkq = Q[k * n + q];
          Q[k * n + p] = c * qkp - s * qkq;
          Q[k * n + q] = s * qkp + c * qkq;
        }
      }
  }
  lam.resize(n);
  for (int i = 0; i < n; ++i) lam[i] = C[i * n + i];
  // S = L^-T Q (back substitution per column)
  S.assign(n * n, 0.0);
  for (int c = 0; c < n; ++c)
    for (int i = n - 1; i >= 0; --i) {
      double s = Q[i * n + c];
      for (int k = i + 1; k < n; ++k) s -= L[k * n + i] * S[k * n + c];
      S[i * n + c] = s / L[i * n + i];
    }
}

void BlockJacobi::setup(const MeshInfo& m, const FE1D& fe, double ip, int precision) {
  EXG_CHECK(m.affine(), EXG_ERR_UNSUPPORTED, "block Jacobi is built for Cartesian meshes");
  EXG_CHECK(precision == EXG_PREC_F32 || precision == EXG_PREC_F64, EXG_ERR_UNSUPPORTED,
            "block Jacobi computes in FP32 or FP64");
  for (int d = 0; d < 3; ++d)
    EXG_CHECK(!m.d.periodic[d] || m.N[d] >= 2, EXG_ERR_UNSUPPORTED,
              "block Jacobi needs two cells along a periodic direction");
  prec = precision;
  n = fe.n;
  n_cells = m.n_cells();
  const double factor = ip * (fe.k + 1.0) * (fe.k + 1.0);
  // tau_c = sum_e (w_low + w_high) / h_e, w = 1 on a non-periodic boundary face, else 1/2
  auto tau_c = [&](const int ci[3]) {
    double t = 0;
    for (int e = 0; e < 3; ++e) {
      const bool lo = ci[e] == 0 && !m.d.periodic[e], hi = ci[e] == m.N[e] - 1 && !m.d.periodic[e];
      t += ((lo ? 1.0 : 0.5) + (hi ? 1.0 : 0.5)) / m.h[e];
    }
    return t;
  };
  // per direction and cell: (kind, tau) of the low and the high face; kind 0 interior/periodic,
  // 1 Dirichlet, 2 Neumann
  using Key = std::tuple<int, int, int, double, double>;  // d, kind_lo, kind_hi, tau_lo, tau_hi
  std::map<Key, int> classes;
  std::vector<Key> keys;
  std::vector<int> cell_cls((size_t)n_cells * 3);
  for (long long c = 0; c < n_cells; ++c) {
    const int ci[3] = {(int)(c % m.N[0]), (int)((c / m.N[0]) % m.N[1]), (int)(c / ((long long)m.N[0] * m.N[1]))};
    const double tc = tau_c(ci);
    for (int d = 0; d < 3; ++d) {
      int kind[2];
      double tau[2];
      for (int side = 0; side < 2; ++side) {
        const bool at_bnd = side == 0 ? ci[d] == 0 : ci[d] == m.N[d] - 1;
        if (!at_bnd || m.d.periodic[d]) {
          int cn[3] = {ci[0], ci[1], ci[2]};
          cn[d] = (ci[d] + (side == 0 ? -1 : 1) + m.N[d]) % m.N[d];
          kind[side] = 0;
          tau[side] = factor * std::max(tc, tau_c(cn));
        } else if (m.d.bc[2 * d + side] == EXG_BC_DIRICHLET) {
          kind[side] = 1;
          tau[side] = factor * tc;
        } else {
          kind[side] = 2;
          tau[side] = 0;
        }
      }
      Key k{d, kind[0], kind[1], tau[0], tau[1]};
      auto it = classes.find(k);
      int id;
      if (it == classes.end()) {
        id = (int)keys.size();
        classes[k] = id;
        keys.push_back(k);
      } else {
        id = it->second;
      }
      cell_cls[(size_t)c * 3 + d] = id;
    }
  }
  n_classes = (int)keys.size();
  std::vector<double> Sall((size_t)n_classes * n * n), Lall((size_t)n_classes * n);
  for (int id = 0; id < n_classes; ++id) {
    const int d = std::get<0>(keys[id]), klo = std::get<1>(keys[id]), khi = std::get<2>(keys[id]);
    const double tlo = std::get<3>(keys[id]), thi = std::get<4>(keys[id]), h = m.h[d];
    std::vector<double> T(n * n), M(n * n), S, lam;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        M[i * n + j] = h * fe.M[i * n + j];
        double t = fe.K[i * n + j] / h;
        // low face (outward normal -e_d): 1/2 (dL_j e0_i + dL_i e0_j) / h + tau e0_i e0_j
        const double wlo = klo == 0 ? 1.0 : (klo == 1 ? 2.0 : 0.0);
        t += wlo * (0.5 * ((i == 0 ? fe.dL[j] : 0.0) + (j == 0 ? fe.dL[i] : 0.0)) / h);
        if (i == 0 && j == 0) t += wlo * tlo;
        // high face (outward normal +e_d): -1/2 (dR_j e_n_i + dR_i e_n_j) / h + tau e_n_i e_n_j
        const double whi = khi == 0 ? 1.0 : (khi == 1 ? 2.0 : 0.0);
        t -= whi * (0.5 * ((i == n - 1 ? fe.dR[j] : 0.0) + (j == n - 1 ? fe.dR[i] : 0.0)) / h);
        if (i == n - 1 && j == n - 1) t += whi * thi;
        T[i * n + j] = t;
      }
    gen_eig(n, T, M, S, lam);
    std::copy(S.begin(), S.end(), Sall.begin() + (size_t)id * n * n);
    std::copy(lam.begin(), lam.end(), Lall.begin() + (size_t)id * n);
  }
  const size_t es = prec == EXG_PREC_F32 ? 4 : 8;
  EXG_CUDA(cudaMalloc(&cls, cell_cls.size() * sizeof(int)));
  EXG_CUDA(cudaMemcpy(cls, cell_cls.data(), cell_cls.size() * sizeof(int), cudaMemcpyHostToDevice));
  EXG_CUDA(cudaMalloc(&S, Sall.size() * es));
  EXG_CUDA(cudaMalloc(&lam, Lall.size() * es));
  if (prec == EXG_PREC_F32) {
    std::vector<float> sf(Sall.begin(), Sall.end()), lf(Lall.begin(), Lall.end());
    EXG_CUDA(cudaMemcpy(S, sf.data(), sf.size() * 4, cudaMemcpyHostToDevice));
    EXG_CUDA(cudaMemcpy(lam, lf.data(), lf.size() * 4, cudaMemcpyHostToDevice));
  } else {
    EXG_CUDA(cudaMemcpy(S, Sall.data(), Sall.size() * 8, cudaMemcpyHostToDevice));
    EXG_CUDA(cudaMemcpy(lam, Lall.data(), Lall.size() * 8, cudaMemcpyHostToDevice));
  }
}

// one 1D sweep along direction D of the cell array u (N^3, x fastest): out = M_D u or M_D^T u
template <int D, int N, bool TRANS, class T>
__device__ __forceinline__ void bj_sweep(const T* __restrict__ Mx, const T* u, T* out, int a, int b) {
  T in[N];
#pragma unroll
  for (int j = 0; j < N; ++j) {
    const int idx = D == 0 ? j + N * (a + N * b) : (D == 1 ? a + N * (j + N * b) : a + N * (b + N * j));
    in[j] = u[idx];
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T s = T(0);
#pragma unroll
    for (int j = 0; j < N; ++j) s += (TRANS ? Mx[j * N + i] : Mx[i * N + j]) * in[j];
    const int idx = D == 0 ? i + N * (a + N * b) : (D == 1 ? a + N * (i + N * b) : a + N * (b + N * i));
    out[idx] = s;
  }
}

// CPB cells per block, N^2 threads per cell (thread (a, b) owns the lines (., a, b), (a, ., b),
// (a, b, .) in turn)
template <int N, int CPB, class T>
__global__ void __launch_bounds__(CPB* N* N) block_jacobi_kernel(const T* __restrict__ src, T* __restrict__ dst,
                                                                 const int* __restrict__ cls,
                                                                 const T* __restrict__ Sg, const T* __restrict__ Lg,
                                                                 long long n_cells) {
  constexpr int N2 = N * N, N3 = N2 * N;
  __shared__ T su[CPB][N3], sv[CPB][N3], sS[CPB][3][N2], sL[CPB][3][N];
  const long long c0 = (long long)blockIdx.x * CPB;
  const int tid = threadIdx.x, lc = tid / N2, l = tid % N2, a = l % N, b = l / N;
  const long long c = c0 + lc;
  const bool active = c < n_cells;
  for (int i = tid; i < CPB * N3; i += CPB * N2) {
    const long long cc = c0 + i / N3;
    su[i / N3][i % N3] = cc < n_cells ? src[c0 * N3 + i] : T(0);
  }
  if (active) {
    for (int d = 0; d < 3; ++d) {
      const int k = cls[c * 3 + d];
      for (int i = l; i < N2; i += N2) sS[lc][d][i] = Sg[(long long)k * N2 + i];
      if (l < N) sL[lc][d][l] = Lg[(long long)k * N + l];
    }
  }
  __syncthreads();
  if (active) bj_sweep<0, N, true, T>(sS[lc][0], su[lc], sv[lc], a, b);  // S_x^T
  __syncthreads();
  if (active) bj_sweep<1, N, true, T>(sS[lc][1], sv[lc], su[lc], a, b);  // S_y^T
  __syncthreads();
  if (active) {
    bj_sweep<2, N, true, T>(sS[lc][2], su[lc], sv[lc], a, b);  // S_z^T, then the eigenvalue scaling
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const int idx = a + N * (b + N * i);
      sv[lc][idx] = sv[lc][idx] / (sL[lc][0][a] + sL[lc][1][b] + sL[lc][2][i]);
    }
  }
  __syncthreads();
  if (active) bj_sweep<2, N, false, T>(sS[lc][2], sv[lc], su[lc], a, b);  // S_z
  __syncthreads();
  if (active) bj_sweep<1, N, false, T>(sS[lc][1], su[lc], sv[lc], a, b);  // S_y
  __syncthreads();
  if (active) bj_sweep<0, N, false, T>(sS[lc][0], sv[lc], su[lc], a, b);  // S_x
  __syncthreads();
  for (int i = tid; i < CPB * N3; i += CPB * N2) {
    const long long cc = c0 + i / N3;
    if (cc < n_cells) dst[c0 * N3 + i] = su[i / N3][i % N3];
  }
}

template <int N, class T>
static void bj_launch(const BlockJacobi& B, const T* src, T* dst, cudaStream_t s) {
  constexpr int CPB = N <= 3 ? 8 : (N <= 5 ? 4 : 2);
  const long long blocks = (B.n_cells + CPB - 1) / CPB;
  block_jacobi_kernel<N, CPB, T><<<(unsigned)blocks, CPB * N * N, 0, s>>>(src, dst, B.cls, (const T*)B.S,
                                                                         (const T*)B.lam, B.n_cells);
  EXG_CUDA(cudaGetLastError());
}

template <class T>
static void bj_apply_t(const BlockJacobi& B, const T* src, T* dst, cudaStream_t s) {
  switch (B.n) {
    case 2: bj_launch<2, T>(B, src, dst, s); break;
    case 3: bj_launch<3, T>(B, src, dst, s); break;
    case 4: bj_launch<4, T>(B, src, dst, s); break;
    case 5: bj_launch<5, T>(B, src, dst, s); break;
    case 6: bj_launch<6, T>(B, src, dst, s); break;
    case 7: bj_launch<7, T>(B, src, dst, s); break;
    case 8: bj_launch<8, T>(B, src, dst, s); break;
    case 9: bj_launch<9, T>(B, src, dst, s); break;
    default: EXG_CHECK(false, EXG_ERR_UNSUPPORTED, "degree must be 1..8");
  }
}

void BlockJacobi::apply(const void* src, void* dst, cudaStream_t s) const {
  if (prec == EXG_PREC_F32)
    bj_apply_t<float>(*this, (const float*)src, (float*)dst, s);
  else
    bj_apply_t<double>(*this, (const double*)src, (double*)dst, s);
}

}  // namespace exg
