// Curved-mesh geometry and kernels (sipg_general.cu).
#pragma once

#include "internal.h"

namespace exg {

// per-cell geometry on the device (precision of the operator)
struct GeneralGeom {
  int precision = EXG_PREC_F64;
  long long n_cells = 0;
  int nq = 0;
  void* cellG = nullptr;        // [cells][nq^3][6]  JxW J^{-1} J^{-T}
  void* face = nullptr;         // [cells][6][nq^2][7] a_own, a_nb, JxW-
  void* ftau = nullptr;         // [cells][6] face penalty tau (k+1)^2 IP max(tau-, tau+)
  long long* fnb = nullptr;     // [cells][6] neighbour, -1 Dirichlet, -2 Neumann
  double* cell_raw = nullptr;   // optional [cells][nq^3][10] G, JxW, x
  double* face_raw = nullptr;   // optional [cells][6][nq^2][16] Jinv, n, JxW, x
  double* tau = nullptr;        // [cells] surface / volume
  int* bc_dev = nullptr;
  bool cell_only = false;       // apply the cell term alone (faces all read as Neumann)
  ~GeneralGeom();
  void build(const MeshInfo& m, const FE1D& fe, double ip, int precision, bool keep_raw, cudaStream_t s);
};

// cells [cell_begin, cell_end) are written (cell_end < 0: to the last cell)
void general_apply(const GeneralGeom& g, const FE1D& fe, const void* src, void* dst, int n_rhs, cudaStream_t s,
                   const PointEpilogue& ep = PointEpilogue(), long long cell_begin = 0, long long cell_end = -1);
void general_diagonal(const GeneralGeom& g, const FE1D& fe, void* out, bool invert, cudaStream_t s);
void general_rhs(const GeneralGeom& g, const FE1D& fe, const double* fq, const double* gq, const double* hq,
                 double* b, cudaStream_t s);
void general_points(const GeneralGeom& g, double* cx, double* fx, long long* ncp, long long* nfp, cudaStream_t s);

}  // namespace exg
