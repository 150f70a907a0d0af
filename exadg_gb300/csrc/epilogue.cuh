// Point-wise vector updates shared by the stand-alone Chebyshev kernel and the operator kernels'
// fused store (PointEpilogue in internal.h).  Both paths evaluate the same expressions in the
// storage type T, so a fused smoother step reproduces the unfused one.
#pragma once

#include "df64.cuh"
#include "internal.h"

namespace exg {

template <class T, class C>
__device__ __forceinline__ T to_storage(C v);
template <>
__device__ __forceinline__ double to_storage<double, double>(double v) { return v; }
template <>
__device__ __forceinline__ float to_storage<float, float>(float v) { return v; }
template <>
__device__ __forceinline__ double to_storage<double, df64>(df64 v) { return join_double(v); }

// Chebyshev recurrence for one entry (modes 1-3 of PointEpilogue), t = (A x)_i
template <class T>
__device__ __forceinline__ T cheb_point(int mode, T xi, T oldi, T bi, T ti, T di, T f1, T f2) {
  T pr = di * (bi - ti);
  if (mode == 1) return xi + f2 * pr;
  if (mode == 2) return (T(1) + f1) * xi + f2 * pr;
  return (T(1) + f1) * xi - f1 * oldi + f2 * pr;
}

// store of the operator value t of DoF i (index into the single right-hand side vectors)
template <class T>
__device__ __forceinline__ void epilogue_store(const PointEpilogue& ep, T* dst, long long i, const T* x, T t) {
  if (ep.mode < 0) {
    dst[i] = t;
    return;
  }
  const T* b = static_cast<const T*>(ep.b);
  T* out = static_cast<T*>(ep.out);
  if (ep.mode == 4) {
    out[i] = b[i] - t;
    return;
  }
  const T* d = static_cast<const T*>(ep.d);
  const T* old = static_cast<const T*>(ep.old);
  T oldi = ep.mode == 3 ? old[i] : T(0);
  out[i] = cheb_point<T>(ep.mode, x[i], oldi, b[i], t, d[i], (T)ep.f1, (T)ep.f2);
}

}  // namespace exg
