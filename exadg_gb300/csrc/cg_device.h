// Device-resident PCG scalars and the one-thread kernels of the graph-driven CG loop.
#pragma once

#include <cuda_runtime.h>

namespace exg {

struct CGDevState {
  double rho, rho_old, alpha, beta, rn, tol;
  int it, max_iter, status, first;  // status: -1 running, 0 converged, 1 iteration cap, 2 non-finite
};

void cg_rho(CGDevState* st, const double* slot, cudaStream_t s);
void cg_p_update(const double* z, double* p, const CGDevState* st, long long n, cudaStream_t s);
void cg_alpha(CGDevState* st, const double* slot, cudaStream_t s);
void cg_check(CGDevState* st, const double* slot, cudaGraphConditionalHandle h, cudaStream_t s);

}  // namespace exg
