// exg_cg_solve_noalloc: the point-Jacobi / unpreconditioned CG solve of exg_cg_solve with every
// work vector taken from one fixed, statically allocated device array instead of cudaMalloc.
//
// Who needs it: callers that must not allocate or free device memory while they run --
// a time loop that keeps kernels of other streams in flight (cudaMalloc / cudaFree synchronise
// the device), and host frameworks whose memory pool owns the whole device.  They give up
// generality: the problem size is capped and calls share one scratch array.
//
// Scratch: kNoallocMaxDofs doubles for each of five work vectors (r, z, p, v, inverse diagonal)
// plus the reduction partials -- about 20 MiB held by every GPU that loads the library until the
// process exits.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <mutex>

#include "host.h"
#include "internal.h"
#include "solver_kernels.h"

namespace exg {

static constexpr long long kNoallocMaxDofs = 1LL << 19;  // 524,288 DoFs
static constexpr int kNoallocRedBlocks = 608;             // partial sums per reduction slot
static constexpr size_t kNoallocVecBytes = (size_t)kNoallocMaxDofs * sizeof(double);
static constexpr size_t kNoallocRedBytes =
    (size_t)kNoallocRedBlocks * Reduction::kSlots * sizeof(double) + Reduction::kSlots * sizeof(double) +
    Reduction::kSlots * sizeof(unsigned int);
static constexpr size_t kNoallocBytes = 5 * kNoallocVecBytes + ((kNoallocRedBytes + 255) / 256) * 256;

// the scratch; host code must not use this symbol as an address (see noalloc_scratch())
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// device address of g_noalloc_scratch on the current device, looked up once per device
static unsigned char* noalloc_scratch() {
  static std::mutex mtx;
  static unsigned char* addr[64] = {nullptr};
  int dev = 0;
  EXG_CUDA(cudaGetDevice(&dev));
  EXG_CHECK(dev >= 0 && dev < 64, EXG_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lock(mtx);
  if (!addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) throw Error{EXG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)};
    addr[dev] = (unsigned char*)p;
  }
  return addr[dev];
}

static double noalloc_read(const Reduction& red, int slot, cudaStream_t s) {
  double v;
  EXG_CUDA(cudaMemcpyAsync(&v, red.out + slot, sizeof(double), cudaMemcpyDeviceToHost, s));
  EXG_CUDA(cudaStreamSynchronize(s));
  return v;
}

static exg_status cg_solve_noalloc(exg_op& op, const exg_cg_desc& d, const double* b, double* x, exg_cg_result& res,
                                   cudaStream_t s) {
  const long long n = op.n_dofs();
  EXG_CHECK(n <= kNoallocMaxDofs, EXG_ERR_INVALID,
            "exg_cg_solve_noalloc: problem has more DoFs than the static scratch holds (524288)");
  EXG_CHECK(d.precond == 0 || d.precond == 1, EXG_ERR_UNSUPPORTED,
            "exg_cg_solve_noalloc supports precond 0 (none) and 1 (point Jacobi)");
  // the diagonal of a continuous operator on a Cartesian mesh is computed through a temporary
  // device table, which would allocate
  EXG_CHECK(!(d.precond == 1 && op.continuous && op.cartesian), EXG_ERR_UNSUPPORTED,
            "exg_cg_solve_noalloc: point Jacobi on a continuous Cartesian operator would allocate");
  unsigned char* base = noalloc_scratch();
  double* r = (double*)(base + 0 * kNoallocVecBytes);
  double* z = (double*)(base + 1 * kNoallocVecBytes);
  double* p = (double*)(base + 2 * kNoallocVecBytes);
  double* v = (double*)(base + 3 * kNoallocVecBytes);
  double* dinv = (double*)(base + 4 * kNoallocVecBytes);
  Reduction red;
  red.partials = (double*)(base + 5 * kNoallocVecBytes);
  red.out = red.partials + (size_t)kNoallocRedBlocks * Reduction::kSlots;
  red.counter = (unsigned int*)(red.out + Reduction::kSlots);
  // the array keeps the previous call's contents: the reduction counters must start at zero
  EXG_CUDA(cudaMemsetAsync(red.counter, 0, Reduction::kSlots * sizeof(unsigned int), s));
  if (d.precond == 1) op.diagonal(dinv, true, s);
  EXG_CUDA(cudaStreamSynchronize(s));
  auto t0 = std::chrono::steady_clock::now();

  // PCG with deal.II SolverCG / ReductionControl semantics (same recurrences as exg_cg_solve)
  dot<double>(x, x, n, red, 0, s);
  bool xzero = noalloc_read(red, 0, s) == 0.0;
  if (xzero) {
    residual<double>(b, nullptr, r, n, red, 1, s);
  } else {
    op.apply(x, v, 1, s);
    residual<double>(b, v, r, n, red, 1, s);
  }
  double rn = std::sqrt(noalloc_read(red, 1, s));
  const double r0 = rn;
  const double tol = std::max(d.abs_tol, d.rel_tol * rn);
  int it = 0, status = std::isfinite(rn) ? (rn <= tol ? 0 : -1) : 2;
  double rho_old = 0;
  while (status < 0) {
    ++it;
    precond_dot<double>(d.precond == 1 ? dinv : nullptr, r, z, n, red, 4, s);
    double rho = noalloc_read(red, 4, s);
    double beta = it == 1 ? 0.0 : rho / rho_old;
    p_update<double>(z, p, beta, it == 1, n, s);
    op.apply(p, v, 1, s);
    dot<double>(p, v, n, red, 2, s);
    double alpha = rho / noalloc_read(red, 2, s);
    xr_update<double>(x, r, p, v, alpha, n, red, 3, s);
    rn = std::sqrt(noalloc_read(red, 3, s));
    rho_old = rho;
    if (!std::isfinite(rn))
      status = 2;
    else if (rn <= tol)
      status = 0;
    else if (it >= d.max_iter)
      status = 1;
  }
  EXG_CUDA(cudaStreamSynchronize(s));
  auto t1 = std::chrono::steady_clock::now();
  res.iterations = it;
  res.converged = status == 0;
  res.r0 = r0;
  res.rn = rn;
  res.rho = it > 0 && r0 > 0 ? std::pow(rn / r0, 1.0 / it) : 0.0;
  res.n10 = (res.rho > 0 && res.rho < 1) ? -10.0 * std::log(10.0) / std::log(res.rho) : 0.0;
  res.seconds = std::chrono::duration<double>(t1 - t0).count();
  if (status == 2) return EXG_ERR_NONFINITE;
  if (status == 1) return EXG_ERR_NOT_CONVERGED;
  return EXG_OK;
}

}  // namespace exg

extern "C" exg_status exg_cg_solve_noalloc(exg_op* op, const exg_cg_desc* desc, const double* b, double* x,
                                           exg_cg_result* result, void* stream) {
  try {
    EXG_CHECK(op && desc && b && x, EXG_ERR_INVALID, "null argument");
    EXG_CHECK(op->precision != EXG_PREC_F32, EXG_ERR_INVALID, "outer CG runs on an FP64 operator");
    exg_cg_result r{};
    exg_status st = exg::cg_solve_noalloc(*op, *desc, b, x, r, (cudaStream_t)stream);
    if (result) *result = r;
    if (st != EXG_OK) exg::set_error(exg_status_string(st));
    return st;
  } catch (const exg::Error& e) {
    exg::set_error(e.msg);
    return e.status;
  } catch (...) {
    exg::set_error("unknown error");
    return EXG_ERR_INVALID;
  }
}
