// Block Jacobi (inverse cell-diagonal blocks) of the SIPG operator on Cartesian meshes by fast
// diagonalisation (block_jacobi.cu).
#pragma once

#include <cuda_runtime.h>

#include "internal.h"

namespace exg {

struct BlockJacobi {
  int prec = EXG_PREC_F64;
  int n = 0;  // nodes per direction (k + 1)
  long long n_cells = 0;
  int n_classes = 0;
  int* cls = nullptr;  // [cells][3] 1D class per direction
  void* S = nullptr;   // [class][n][n] generalised eigenvectors (S^T M S = I)
  void* lam = nullptr; // [class][n] eigenvalues
  BlockJacobi() = default;
  BlockJacobi(const BlockJacobi&) = delete;
  BlockJacobi& operator=(const BlockJacobi&) = delete;
  ~BlockJacobi();
  // synchronous (allocations and copies): call before any stream capture
  void setup(const MeshInfo& m, const FE1D& fe, double ip, int precision);
  // dst = blockdiag(A)^-1 src (precision of the set-up)
  void apply(const void* src, void* dst, cudaStream_t s) const;
};

}  // namespace exg
