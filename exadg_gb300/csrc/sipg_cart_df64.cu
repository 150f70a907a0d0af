// FP32-pair (df64) instantiation of the affine SIPG apply kernels (templates in sipg_cartesian.cuh); one
// translation unit per arithmetic so the variants compile in parallel.
#include "sipg_cartesian.cuh"

namespace exg {
void cart_apply_df64(const CartHost& h, const void* src, void* dst, int n_rhs, int cpb, cudaStream_t s,
                     const PointEpilogue& ep) {
  apply_prec<double, df64>(h, src, dst, n_rhs, cpb, s, ep);
}
}  // namespace exg
