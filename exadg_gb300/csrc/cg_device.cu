// Device-resident PCG iteration (deal.II SolverCG with ReductionControl,
// solvers/iterative_solvers_dealii_wrapper.h:136-221): the scalars rho, beta, alpha and the
// residual norm stay in device memory and the convergence test runs in a one-thread kernel that
// sets the condition of a CUDA-graph WHILE node, so an entire solve is one graph launch with no
// host round trip per iteration.  The arithmetic (FP64 reductions, the order of the updates, the
// stopping test after each residual update) is that of the host-driven loop in host.cpp.
#include <cuda_runtime.h>

#include <cmath>

#include "cg_device.h"
#include "internal.h"

namespace exg {

static constexpr int kBlocks = 608;  // 4 x 152 SMs, as the reduction kernels
static constexpr int kThreads = 256;

// rho = r.z (from the reduction slot); beta = rho / rho_old after the first iteration
__global__ void cg_rho_kernel(CGDevState* st, const double* __restrict__ slot) {
  const double rho = *slot;
  st->first = st->it == 0 ? 1 : 0;
  st->beta = st->it == 0 ? 0.0 : rho / st->rho_old;
  st->rho = rho;
}

__global__ void cg_p_update_kernel(const double* __restrict__ z, double* __restrict__ p,
                                   const CGDevState* __restrict__ st, long long n) {
  const double beta = st->beta;
  const bool first = st->first != 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = first ? z[i] : z[i] + beta * p[i];
}

// alpha = rho / p.v
__global__ void cg_alpha_kernel(CGDevState* st, const double* __restrict__ slot) { st->alpha = st->rho / *slot; }

// convergence test after the residual update: |r| <= tol, iteration cap, non-finite residual; the
// WHILE node runs the next iteration only while the status stays 'running'
__global__ void cg_check_kernel(CGDevState* st, const double* __restrict__ slot, cudaGraphConditionalHandle h) {
  const double rn = sqrt(*slot);
  st->rn = rn;
  st->it += 1;
  st->rho_old = st->rho;
  int status = -1;
  if (!isfinite(rn))
    status = 2;
  else if (rn <= st->tol)
    status = 0;
  else if (st->it >= st->max_iter)
    status = 1;
  st->status = status;
  cudaGraphSetConditional(h, status < 0 ? 1u : 0u);
}

void cg_rho(CGDevState* st, const double* slot, cudaStream_t s) {
  cg_rho_kernel<<<1, 1, 0, s>>>(st, slot);
  EXG_CUDA(cudaGetLastError());
}
void cg_p_update(const double* z, double* p, const CGDevState* st, long long n, cudaStream_t s) {
  cg_p_update_kernel<<<kBlocks, kThreads, 0, s>>>(z, p, st, n);
  EXG_CUDA(cudaGetLastError());
}
void cg_alpha(CGDevState* st, const double* slot, cudaStream_t s) {
  cg_alpha_kernel<<<1, 1, 0, s>>>(st, slot);
  EXG_CUDA(cudaGetLastError());
}
void cg_check(CGDevState* st, const double* slot, cudaGraphConditionalHandle h, cudaStream_t s) {
  cg_check_kernel<<<1, 1, 0, s>>>(st, slot, h);
  EXG_CUDA(cudaGetLastError());
}

}  // namespace exg
