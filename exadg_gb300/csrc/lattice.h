// Continuous Q_k levels of cphMG on Cartesian meshes: the Laplace operator on the node lattice
// and the transfers into, between and out of continuous levels (lattice.cu).
//
// FE_Q(k) with Gauss-Lobatto support points on a box of N[0] x N[1] x N[2] equal cells has
// n_d = N_d k + 1 nodes per direction (N_d k when d is periodic), numbered x fastest.  On equal
// box cells the cell-integral Laplacian with k+1 Gauss points is exactly the Kronecker sum
// A = K_x M_y M_z + M_x K_y M_z + M_x M_y K_z of assembled 1D mass and stiffness matrices
// (LaplaceOperator::do_cell_integral, poisson/spatial_discretization/laplace_operator.cpp; the
// operator of a continuous level has no face integrals, operators/operator_base.cpp:264-310).
// Row g of a 1D matrix has the band g-k..g+k; its entries depend only on the row type: g mod k
// (0 = a vertex shared by two cells), k = first node of a bounded line, k+1 = its last node.
// Constrained nodes (nodes on Dirichlet sides; node 0 of a singular operator,
// solvers_and_preconditioners/multigrid/constraints.h:130-197) are read as zero and keep
// dst = src (identity rows, operator_base.cpp:299-308).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "internal.h"

namespace exg {

constexpr int LAT_KMAX = 8;

// which lattice nodes are constrained (kernel-side, by coordinates)
struct LatticeMask {
  int n[3];
  int periodic[3];
  int dirichlet[6];
  int pin_first;
};

struct LatticeHost {
  int N[3], k;
  LatticeMask mask;
  double h[3];
  // band coefficients [dir][0 = mass, 1 = stiffness][row type 0..k+1][o + k], o = -k..k
  std::vector<double> coef;
  long long size() const { return (long long)mask.n[0] * mask.n[1] * mask.n[2]; }
};

// lattice of the mesh m at degree k (singular: pin node 0)
void make_lattice(const MeshInfo& m, int k, bool singular, LatticeHost& L);
bool lattice_constrained(const LatticeMask& m, int gx, int gy, int gz);

// dst = A src (precision EXG_PREC_F32 / EXG_PREC_F64), the store through the point epilogue
void lattice_apply(LatticeHost& L, int precision, const void* src, void* dst, cudaStream_t s,
                   const PointEpilogue& ep = PointEpilogue());
void lattice_diagonal(LatticeHost& L, int precision, void* diag, bool invert, cudaStream_t s);
// uploads the unit-cell band tables to the current device once (synchronous: call before any
// stream capture)
void lattice_prepare(LatticeHost& L, int precision);

// Curved meshes: the continuous operator is the DG operator's cell term (a GeneralGeom whose faces
// all read as Neumann) between a masked gather of the lattice into the DG layout and a sum back
// per node.  lattice_to_dg: dg = gather(lat), constrained nodes as zero.  dg_to_lattice_apply:
// t = sum of the DG entries at each node, src on constrained nodes, stored through the point
// epilogue.  dg_to_lattice_diagonal: the same sum of the cell-term diagonals, 1 on constrained
// nodes, optionally inverted.
void lattice_to_dg(const LatticeHost& L, int precision, const void* lat, void* dg, cudaStream_t s);
void dg_to_lattice_apply(const LatticeHost& L, int precision, const void* dg, const void* src, void* dst,
                         const PointEpilogue& ep, cudaStream_t s);
void dg_to_lattice_diagonal(const LatticeHost& L, int precision, const void* dg, void* diag, bool invert,
                            cudaStream_t s);

// transfer between level l-1 (continuous) and level l (continuous, or the discontinuous level of
// the same mesh and degree: the c-transfer)
struct LatticeTransfer {
  bool to_dg = false;
  int prec = EXG_PREC_F32;
  LatticeMask mc{}, mf{};
  int Nc[3] = {0, 0, 0}, kc = 1, kf = 1;  // c-transfer: the DG level's cells and degree
  // per direction: prolongation rows (fine nodes x wp entries) and restriction rows (coarse nodes
  // x wr entries), column indices and values in the level precision
  int wp[3] = {0, 0, 0}, wr[3] = {0, 0, 0};
  int* pcol[3] = {nullptr, nullptr, nullptr};
  int* rcol[3] = {nullptr, nullptr, nullptr};
  void* pval[3] = {nullptr, nullptr, nullptr};
  void* rval[3] = {nullptr, nullptr, nullptr};
  void* scratch[2] = {nullptr, nullptr};
  LatticeTransfer() = default;
  LatticeTransfer(const LatticeTransfer&) = delete;
  LatticeTransfer& operator=(const LatticeTransfer&) = delete;
  ~LatticeTransfer();
  // continuous coarse -> continuous fine (p: same cells; h: fine cells = 2 x coarse cells)
  void setup(const LatticeHost& coarse, const LatticeHost& fine, int precision);
  // continuous coarse -> discontinuous fine of the same mesh and degree
  void setup_dg(const LatticeHost& coarse, int precision);
  void prolongate_add(const void* coarse, void* fine, cudaStream_t s) const;
  void restrict_add(const void* fine, void* coarse, cudaStream_t s) const;
};

}  // namespace exg
