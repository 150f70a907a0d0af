// Declarations of the solver-side kernels (solver_kernels.cu).
#pragma once

#include <cuda_runtime.h>

namespace exg {

// device scratch for deterministic FP64 reductions; result of slot s lands in out[s]
struct Reduction {
  static constexpr int kSlots = 8;
  double* partials = nullptr;
  double* out = nullptr;
  unsigned int* counter = nullptr;
  static Reduction create();
  void destroy();
};

template <class T> void dot(const T* x, const T* y, long long n, Reduction& red, int slot, cudaStream_t s);
template <class T> void residual(const T* b, const T* v, T* r, long long n, Reduction& red, int slot, cudaStream_t s);
template <class T> void precond_dot(const T* d, const T* r, T* z, long long n, Reduction& red, int slot, cudaStream_t s);
template <class T> void p_update(const T* z, T* p, double beta, bool first, long long n, cudaStream_t s);
template <class T>
void xr_update(T* x, T* r, const T* p, const T* v, double alpha, long long n, Reduction& red, int slot, cudaStream_t s);
void xr_update_dev(double* x, double* r, const double* p, const double* v, const double* alpha, long long n,
                   Reduction& red, int slot, cudaStream_t s);
template <class T>
void chebyshev_update(int mode, T* x, T* old, const T* b, const T* t, const T* d, double f1, double f2, long long n,
                      cudaStream_t s);
template <class T> void rsub(const T* b, T* t, long long n, cudaStream_t s);

struct TransferParams {
  int is_h;
  int nf, nc;
  int Nf[3], Nc[3];
  double P[2][81];  // 1D prolongation (nf x nc), child 0/1 for h-transfer
};
template <class T> void prolongate_add(const TransferParams& P, const T* coarse, T* fine, cudaStream_t s);
template <class T> void restrict_add(const TransferParams& P, const T* fine, T* coarse, cudaStream_t s);

template <class T, class CT>
void coarse_cg(const CT* A, const CT* invd, const T* rhs, T* x, CT* xstate, int n, double rel_tol, double abs_tol,
               int max_iter, int singular, long long* its, cudaStream_t s);
template <class T, class CT> void coarse_cg_prepare(int n);
template <class T> void identity(T* e, int n, cudaStream_t s);

}  // namespace exg
