// Internal declarations shared by the host library and the CUDA translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/exadg_gb300.h"

namespace exg {

// ------------------------------------------------------------------------------------------
// error handling: every C entry point returns a status and records a message
// ------------------------------------------------------------------------------------------
void set_error(const std::string& msg);
struct Error {
  exg_status status;
  std::string msg;
};
#define EXG_CUDA(call)                                                                       \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      throw ::exg::Error{EXG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
  } while (0)
#define EXG_CHECK(cond, status, msg)                    \
  do {                                                  \
    if (!(cond)) throw ::exg::Error{(status), (msg)}; \
  } while (0)

// ------------------------------------------------------------------------------------------
// 1D finite element tables on [0,1]: FE_DGQ(k) on Gauss-Lobatto nodes, Gauss quadrature
// ------------------------------------------------------------------------------------------
struct FE1D {
  int k, n, nq;
  std::vector<double> gl;      // n Gauss-Lobatto nodes
  std::vector<double> gq, gw;  // nq Gauss points / weights
  std::vector<double> S, D;    // nq x n values / derivatives of the Lagrange basis at gq
  std::vector<double> M, K;    // n x n reference mass / stiffness
  std::vector<double> dL, dR;  // basis derivatives at 0 and 1
  void init(int degree, int n_q);
};
std::vector<double> gauss_lobatto(int n);
void gauss(int n, std::vector<double>& x, std::vector<double>& w);
double lagrange(const std::vector<double>& z, int i, double x);
double lagrange_d(const std::vector<double>& z, int i, double x);

// ------------------------------------------------------------------------------------------
// mesh
// ------------------------------------------------------------------------------------------
struct MeshInfo {
  exg_mesh_desc d;
  int N[3];
  double h[3];
  bool affine() const { return d.deform_amp == 0.0; }
  long long n_cells() const { return (long long)N[0] * N[1] * N[2]; }
};

// kernel-side view of a structured mesh
struct CartMesh {
  int N[3];
  int periodic[3];
  int bc[6];  // 0 Dirichlet, 1 Neumann
  long long n_cells;
  long long n_dofs;
  long long cell_begin, cell_end;  // cells written by a launch (row kernels): [cell_begin, cell_end)
};

// penalty data for Cartesian meshes: tau_c = sum_e (wL_e + wR_e) / h_e
struct CartPenalty {
  double inv_h[3];
  double factor;  // (k+1)^2 * IP
};

// ------------------------------------------------------------------------------------------
// Cartesian launchers (sipg_cartesian.cu)
// ------------------------------------------------------------------------------------------
struct CartHost {
  int n;
  double M[81];
  double B[3][81];
  double sdL[3][9], sdR[3][9];
  double A[3];
  CartPenalty pen;
  double tauA[3][64];  // A_d * tau_c * (k+1)^2 IP per boundary class of the cell (see cell_class)
  CartMesh mesh;
};
void build_cart_host(const MeshInfo& m, const FE1D& fe, double ip, CartHost& out);

// Point-wise update fused into the operator's store: with t = (A x)_i for the DoF i the kernel
// writes out_i instead of t (vectors in the operator's storage type, one right-hand side):
//   mode -1: out = dst, out_i = t                           (plain apply)
//   mode  1: out_i = x_i + f2 d_i (b_i - t)                 (Chebyshev step, first update)
//   mode  2: out_i = (1 + f1) x_i + f2 d_i (b_i - t)        (second update after a zero start)
//   mode  3: out_i = (1 + f1) x_i - f1 old_i + f2 d_i (b_i - t)
//   mode  4: out_i = b_i - t                                (residual)
// out may alias old (each index is read and then written by the same thread); it must not alias x.
struct PointEpilogue {
  int mode = -1;
  const void* old = nullptr;
  const void* b = nullptr;
  const void* d = nullptr;
  void* out = nullptr;
  double f1 = 0, f2 = 0;
};

// precision: EXG_PREC_F64 / EXG_PREC_F32 / EXG_PREC_F64E; cpb = cells per block (0 = default)
void cart_apply(const CartHost& h, int precision, const void* src, void* dst, int n_rhs, int cpb,
                cudaStream_t s, const PointEpilogue& ep = PointEpilogue());
void cart_diagonal(const CartHost& h, int precision, void* diag, bool invert, cudaStream_t s);
std::vector<int> cart_cpb_options(int n, int precision);

// ------------------------------------------------------------------------------------------
// vector kernels (vec_ops.cu)
// ------------------------------------------------------------------------------------------
void vec_copy_convert(const void* src, int src_prec, void* dst, int dst_prec, long long n, cudaStream_t s);
void vec_fill(void* x, int prec, double v, long long n, cudaStream_t s);
void device_fma_peaks(double* f64_tflops, double* f32_tflops, cudaStream_t s);
// raises a kernel's dynamic shared-memory limit to at least `bytes` on the current device (the
// attribute is per device; thread-safe, a no-op once set)
void ensure_smem_attr(const void* kernel, int bytes);

}  // namespace exg
