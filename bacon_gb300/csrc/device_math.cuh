// Device arithmetic policies and the deterministic fourth root.
//
// ExactOps rounds every product, sum and quotient separately (no fused
// multiply-add), so a kernel written with it executes the same IEEE-754
// operation sequence as the reference's Rust code, which LLVM never
// contracts.  FmaOps lets nvcc contract mul+add pairs.
#pragma once

#include <cstdint>

namespace bacon {

struct ExactOps {
  static constexpr bool kExact = true;
  __device__ __forceinline__ static double mul(double a, double b) { return __dmul_rn(a, b); }
  __device__ __forceinline__ static double add(double a, double b) { return __dadd_rn(a, b); }
  __device__ __forceinline__ static double sub(double a, double b) { return __dsub_rn(a, b); }
  __device__ __forceinline__ static double div(double a, double b) { return __ddiv_rn(a, b); }
  __device__ __forceinline__ static double sqrt(double a) { return __dsqrt_rn(a); }
  // a + b*c, as "a += b * c" with two roundings.
  __device__ __forceinline__ static double axpy(double a, double b, double c) {
    return __dadd_rn(a, __dmul_rn(b, c));
  }
};

struct FmaOps {
  static constexpr bool kExact = false;
  __device__ __forceinline__ static double mul(double a, double b) { return a * b; }
  __device__ __forceinline__ static double add(double a, double b) { return a + b; }
  __device__ __forceinline__ static double sub(double a, double b) { return a - b; }
  __device__ __forceinline__ static double div(double a, double b) { return __ddiv_rn(a, b); }
  __device__ __forceinline__ static double sqrt(double a) { return __dsqrt_rn(a); }
  __device__ __forceinline__ static double axpy(double a, double b, double c) {
    return __fma_rn(b, c, a);
  }
};

// Bit mask of the non-finite components of v (bit d set if v[d] is +-inf or
// NaN).  Integer operations on the high word only: no FP64 pipe use.
template <int D>
__device__ __forceinline__ uint32_t nonfinite_mask(const double (&v)[D]) {
  uint32_t m = 0;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const uint32_t hi = static_cast<uint32_t>(__double2hiint(v[d]));
    m |= static_cast<uint32_t>((hi & 0x7ff00000u) == 0x7ff00000u) << d;
  }
  return m;
}

// One correction of r toward the correctly rounded x^(1/4): the residual
// x - r^4 is formed in double-double and compared with the distance to the
// neighbouring rounding midpoints (times 4 r^3).  The same operation
// sequence runs in the CPU restatement used by the tests.
__device__ __forceinline__ double qrt_fix(double x, double r) {
  const double p_hi = __dmul_rn(r, r);
  const double p_lo = __fma_rn(r, r, -p_hi);
  const double q_hi = __dmul_rn(p_hi, p_hi);
  double q_lo = __fma_rn(p_hi, p_hi, -q_hi);
  q_lo = __fma_rn(__dmul_rn(2.0, p_hi), p_lo, q_lo);
  const double res = __dsub_rn(__dsub_rn(x, q_hi), q_lo);
  const unsigned long long rb = static_cast<unsigned long long>(__double_as_longlong(r));
  const unsigned long long e = (rb >> 52) & 0x7ffull;
  const double half_ulp = __longlong_as_double(static_cast<long long>((e - 53ull) << 52));
  const double thr_up = __dmul_rn(__dmul_rn(4.0, half_ulp), __dmul_rn(p_hi, r));
  const double thr_dn = ((rb & 0x000fffffffffffffull) == 0ull) ? __dmul_rn(0.5, thr_up) : thr_up;
  if (res > thr_up) return __longlong_as_double(static_cast<long long>(rb + 1ull));
  if (res < -thr_dn) return __longlong_as_double(static_cast<long long>(rb - 1ull));
  return r;
}

// x^(1/4) for the step-size controller (the reference evaluates
// (tol/err).powf(1/4), src/ivp/rk.rs:400-401).  Exact for the special values
// pow() defines on this domain: +0 -> +0, +inf -> +inf, NaN -> NaN.
__device__ __forceinline__ double qrt(double x) {
  if (!(x > 0.0)) return (x == 0.0) ? 0.0 : __longlong_as_double(0x7ff8000000000000ll);
  if (__double2hiint(x) == 0x7ff00000 && __double2loint(x) == 0) return x;  // +inf
  double s = 1.0;
  if (x > 0x1p400) {
    x = __dmul_rn(x, 0x1p-800);
    s = 0x1p200;
  } else if (x < 0x1p-400) {
    x = __dmul_rn(x, 0x1p800);
    s = 0x1p-200;
  }
  // sqrt(sqrt(x)) is within one ulp of x^(1/4): the inner rounding moves the
  // root by at most 2^-54 relative (half an ulp at the top of a binade) and
  // the outer rounding by half an ulp.  One correction therefore reaches the
  // correctly rounded value.
  const double r = qrt_fix(x, __dsqrt_rn(__dsqrt_rn(x)));
  return __dmul_rn(r, s);
}

}  // namespace bacon
