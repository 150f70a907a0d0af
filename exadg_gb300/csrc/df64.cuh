// Compute-type traits for the operator kernels: native double, native float, and df64 -- an
// unevaluated sum of two floats ("double-float", Dekker 1971; error-free transformations TwoSum
// (Knuth) and TwoProd via FMA).  GB300 executes FP32 FMAs at ~60x the FP64 rate, so df64
// arithmetic (about 12 FP32 operations per multiply-add, ~2^-48 relative precision) is the fast
// way to reach FP64-level accuracy (<= 1e-12 relative) on this part.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace exg {

struct df64 {
  float hi, lo;
  df64() = default;
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr df64(int v) : hi((float)v), lo(0.0f) {}
};

// ---------------------------------------------------------------- coefficient conversion (host)
template <class C>
__host__ __device__ inline C coef_from_double(double v);
template <>
__host__ __device__ inline double coef_from_double<double>(double v) { return v; }
template <>
__host__ __device__ inline float coef_from_double<float>(double v) { return (float)v; }
template <>
__host__ __device__ inline df64 coef_from_double<df64>(double v) {
  float h = (float)v;
  float l = (float)(v - (double)h);
  return df64(h, l);
}

__host__ __device__ inline double coef_to_double(double v) { return v; }
__host__ __device__ inline double coef_to_double(float v) { return (double)v; }
__host__ __device__ inline double coef_to_double(df64 v) { return (double)v.hi + (double)v.lo; }

// ---------------------------------------------------------------- native types
__device__ __forceinline__ double fmadd(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmadd(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double neg(double a) { return -a; }
__device__ __forceinline__ float neg(float a) { return -a; }

// ---------------------------------------------------------------- df64 arithmetic
// double -> df64 without FP64 arithmetic: the high word keeps the leading 24 significand bits
// (truncation), the low word the remaining 29 bits rounded to 24.  Exact to 2^-48 relative for
// |x| in [2^-74, 2^127]; smaller entries keep the high word only, |x| < 2^-126 flushes to zero.
__device__ __forceinline__ df64 split_double(double x) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const unsigned int sign = (unsigned int)(bits >> 32) & 0x80000000u;
  const int e = (int)((bits >> 52) & 0x7FF);
  const int fe = e - 896;  // float biased exponent
  if (fe <= 0) return df64(0.0f, 0.0f);
  if (fe >= 255) return df64(__int_as_float((int)(sign | 0x7F800000u)), 0.0f);
  const unsigned int hib = sign | ((unsigned int)fe << 23) | (unsigned int)((bits >> 29) & 0x7FFFFFu);
  const unsigned int low = (unsigned int)(bits & 0x1FFFFFFFu);
  const int le = e - 948;  // exponent of one unit of the low 29 bits, biased
  float lo = 0.0f;
  if (le > 0) lo = __uint_as_float(__float_as_uint(__uint2float_rn(low) * __int_as_float(le << 23)) | sign);
  return df64(__uint_as_float(hib), lo);
}

__device__ __forceinline__ double join_double(df64 v) { return (double)v.hi + (double)v.lo; }

__device__ __forceinline__ df64 two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float err = (a - (s - bb)) + (b - bb);
  return df64(s, err);
}
__device__ __forceinline__ df64 fast_two_sum(float a, float b) {
  float s = a + b;
  float err = b - (s - a);
  return df64(s, err);
}

// c + a*b, result not renormalised (hi carries the rounded leading part, lo the rest)
__device__ __forceinline__ df64 fmadd(df64 a, df64 b, df64 c) {
  float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  df64 s = two_sum(c.hi, p);
  return df64(s.hi, s.lo + (c.lo + e));
}
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + df64(-b.hi, -b.lo); }
__device__ __forceinline__ df64 neg(df64 a) { return df64(-a.hi, -a.lo); }

// small exactly representable constants in the compute type
template <class C>
__host__ __device__ inline C cconst(double v);
template <>
__host__ __device__ inline double cconst<double>(double v) { return v; }
template <>
__host__ __device__ inline float cconst<float>(double v) { return (float)v; }
template <>
__host__ __device__ inline df64 cconst<df64>(double v) { return df64((float)v, 0.0f); }

// ---------------------------------------------------------------- loads / stores
template <class C, class T>
__device__ __forceinline__ C load_as(const T* p);
template <>
__device__ __forceinline__ double load_as<double, double>(const double* p) { return __ldg(p); }
template <>
__device__ __forceinline__ float load_as<float, float>(const float* p) { return __ldg(p); }
template <>
__device__ __forceinline__ df64 load_as<df64, double>(const double* p) { return split_double(__ldg(p)); }

template <class T, class C>
__device__ __forceinline__ void store_as(T* p, C v);
template <>
__device__ __forceinline__ void store_as<double, double>(double* p, double v) { *p = v; }
template <>
__device__ __forceinline__ void store_as<float, float>(float* p, float v) { *p = v; }
template <>
__device__ __forceinline__ void store_as<double, df64>(double* p, df64 v) { *p = join_double(v); }

// bytes of the per-cell face header (neighbour index, penalty, kind) in shared memory, rounded to 16
template <class C>
__host__ __device__ constexpr size_t smem_head_bytes(int cpb) {
  return ((size_t)cpb * 6 * (sizeof(C) + 2 * sizeof(int)) + 15) / 16 * 16;
}

}  // namespace exg
