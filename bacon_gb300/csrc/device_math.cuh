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

// Compares off the FP64 pipe.  The left operand is a norm, a ratio of
// norms or a step size: non-negative (never -0) or NaN; the right one is
// a positive tolerance, step bound or constant, or NaN.  For such values the
// integer order of the bit patterns is the numeric order, and with the NaN
// cases excluded explicitly each helper returns exactly the IEEE result.
constexpr unsigned long long kInfBits = 0x7ff0000000000000ull;
__device__ __forceinline__ unsigned long long nn_bits(double x) {
  return static_cast<unsigned long long>(__double_as_longlong(x));
}
__device__ __forceinline__ bool nn_le(double a, double b) {  // a <= b
  return nn_bits(a) <= nn_bits(b) && nn_bits(b) <= kInfBits;
}
__device__ __forceinline__ bool nn_lt(double a, double b) {  // a < b
  return nn_bits(a) < nn_bits(b) && nn_bits(b) <= kInfBits;
}
__device__ __forceinline__ bool nn_ge(double a, double b) {  // a >= b
  return nn_bits(a) >= nn_bits(b) && nn_bits(a) <= kInfBits && nn_bits(b) <= kInfBits;
}
__device__ __forceinline__ bool nn_gt(double a, double b) {  // a > b
  return nn_bits(a) > nn_bits(b) && nn_bits(a) <= kInfBits && nn_bits(b) <= kInfBits;
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
  const long long e = static_cast<long long>((rb >> 52) & 0x7ffull);
  // thr_up = 4 * (half an ulp of r) * p_hi * r = RN(p_hi r) * 2^(e - 1074), e
  // the biased exponent of r.  After qrt's range split r is in [2^-100,
  // 2^100], so the power-of-two scaling stays in the normal range: it is
  // exact, and done on the exponent field; so is the halving of thr_dn.
  const double thr_up = __longlong_as_double(__double_as_longlong(__dmul_rn(p_hi, r)) + (e - 1074) * (1ll << 52));
  const double thr_dn =
      ((rb & 0x000fffffffffffffull) == 0ull) ? __longlong_as_double(__double_as_longlong(thr_up) - (1ll << 52)) : thr_up;
  // res > thr_up and res < -thr_dn on the bit patterns (res finite of either
  // sign, the thresholds positive normal): a signed compare orders res
  // against a positive value, and res < -thr_dn is a negative res of larger
  // magnitude
  const long long resb = __double_as_longlong(res);
  if (resb > __double_as_longlong(thr_up)) return __longlong_as_double(static_cast<long long>(rb + 1ull));
  if (resb < 0 && static_cast<unsigned long long>(resb & 0x7fffffffffffffffll) > nn_bits(thr_dn))
    return __longlong_as_double(static_cast<long long>(rb - 1ull));
  return r;
}

// x^(1/4) for the step-size controller (the reference evaluates
// (tol/err).powf(1/4), src/ivp/rk.rs:400-401).  Exact for the special values
// pow() defines on this domain: +0 -> +0, +inf -> +inf, NaN -> NaN.
__device__ __forceinline__ double qrt(double x) {
  // the special cases and the range split on the bit pattern (integer compares)
  const long long xb = __double_as_longlong(x);
  if (!(xb > 0 && xb <= static_cast<long long>(kInfBits)))  // !(x > 0): zeros, negatives, NaN
    return ((xb & 0x7fffffffffffffffll) == 0) ? 0.0 : __longlong_as_double(0x7ff8000000000000ll);
  if (xb == static_cast<long long>(kInfBits)) return x;  // +inf
  double s = 1.0;
  bool scaled = false;
  if (xb > 0x58f0000000000000ll) {  // x > 2^400
    x = __dmul_rn(x, 0x1p-800);
    s = 0x1p200;
    scaled = true;
  } else if (xb < 0x26f0000000000000ll) {  // x < 2^-400
    x = __dmul_rn(x, 0x1p800);
    s = 0x1p-200;
    scaled = true;
  }
  // sqrt(sqrt(x)) is within one ulp of x^(1/4): the inner rounding moves the
  // root by at most 2^-54 relative (half an ulp at the top of a binade) and
  // the outer rounding by half an ulp.  One correction therefore reaches the
  // correctly rounded value.
  const double r = qrt_fix(x, __dsqrt_rn(__dsqrt_rn(x)));
  return scaled ? __dmul_rn(r, s) : r;
}

// One ulp-step correction of r ~ (z + adj)^(1/N), z in [1, 2^N), r in [1, 2):
// the residual z + adj - r^N in double-double against N r^(N-1) times half an
// ulp (the first-order distance to the rounding midpoints).
template <int N>
__device__ __forceinline__ double rootn_fix(double z, double r, double adj) {
  const double r2 = __dmul_rn(r, r);
  const double r2lo = __fma_rn(r, r, -r2);
  double hi, lo, deriv;
  if constexpr (N == 3) {
    hi = __dmul_rn(r2, r);
    lo = __fma_rn(r2lo, r, __fma_rn(r2, r, -hi));
    deriv = __dmul_rn(3.0, r2);
  } else {
    const double r4 = __dmul_rn(r2, r2);
    const double r4lo = __fma_rn(__dmul_rn(2.0, r2), r2lo, __fma_rn(r2, r2, -r4));
    hi = __dmul_rn(r4, r);
    lo = __fma_rn(r4lo, r, __fma_rn(r4, r, -hi));
    deriv = __dmul_rn(5.0, r4);
  }
  const double res = __dadd_rn(__dsub_rn(__dsub_rn(z, hi), lo), adj);
  const unsigned long long rb = static_cast<unsigned long long>(__double_as_longlong(r));
  const unsigned long long e = (rb >> 52) & 0x7ffull;
  const double half_ulp = __longlong_as_double(static_cast<long long>((e - 53ull) << 52));
  const double thr_up = __dmul_rn(half_ulp, deriv);
  const double thr_dn = ((rb & 0x000fffffffffffffull) == 0ull) ? __dmul_rn(0.5, thr_up) : thr_up;
  if (res > thr_up) return __longlong_as_double(static_cast<long long>(rb + 1ull));
  if (res < -thr_dn) return __longlong_as_double(static_cast<long long>(rb - 1ull));
  return r;
}

// x^RN(1/N) for N = 3 or 5: what the reference's Adams controller evaluates,
// (tol / (2 err)).powf(N.recip()) (src/ivp/adams.rs:527-528, :551-552).  The
// rounded exponent is 1/N + delta (delta = +2^-54/5, -2^-54/3), so the value
// is the true root times 1 + delta ln x.  Exponent split x = 2^(Nq) z with z
// in [1, 2^N), an FP32 first guess, two Newton steps and an ulp-step
// correction give the true root; ln x (exponent plus a
// short atanh series, relative error < 1e-5) moves it by the factor
// 1 + delta ln x, and a second ulp-step correction on the residual of the
// radicand z (1 + N delta ln x) rounds it.  From the first correction on, the
// same operation sequence as the CPU oracle's oracle_rootn; correctly rounded
// except within ~2^-50 ulp of a midpoint.  0 -> 0, inf -> inf, negative or
// NaN -> NaN (as pow).
template <int N>
__device__ __forceinline__ double rootn(double x) {
  static_assert(N == 3 || N == 5, "orders 3 and 5");
  if (!(x > 0.0)) return (x == 0.0) ? 0.0 : __longlong_as_double(0x7ff8000000000000ll);
  if (__double2hiint(x) == 0x7ff00000 && __double2loint(x) == 0) return x;  // +inf
  double s = 1.0;
  int shift = 0;
  if (x < 0x1p-1000) {
    x = __dmul_rn(x, N == 3 ? 0x1p900 : 0x1p1000);
    s = (N == 3) ? 0x1p-300 : 0x1p-200;
    shift = (N == 3) ? 900 : 1000;
  }
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const int e = static_cast<int>(b >> 52) - 1023;
  int q = e / N, rem = e % N;
  if (rem < 0) {
    rem += N;
    q -= 1;
  }
  const double z = __longlong_as_double(
      static_cast<long long>((b & 0x000fffffffffffffull) | (static_cast<unsigned long long>(1023 + rem) << 52)));
  // The true root z^(1/N) to within one ulp, then the ulp-step correction.
  // First guess from the FP32 special-function units (log2, exp2: relative
  // error ~2^-21), then two Newton steps in FP64 whose divisor is an FP32
  // reciprocal: the error goes 2^-21 -> ~2^-41 -> the rounding of the last
  // step plus ~0.15 ulp from the rounded y^N, so y is the correctly rounded
  // root or a neighbour, which is all rootn_fix needs.  (The CPU oracle
  // starts from a bit-pattern guess with five divided Newton steps; the two
  // agree after rootn_fix except within ~2^-50 ulp of a rounding midpoint.)
  // The dependent chain is a third of five divided steps, which matters
  // because a warp pays for the root whenever any of its lanes needs one.
  double y = static_cast<double>(exp2f(__fmul_rn(log2f(__double2float_rn(z)), 1.0f / static_cast<float>(N))));
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    double ym1 = y;
#pragma unroll
    for (int k = 2; k < N; ++k) ym1 = __dmul_rn(ym1, y);
    const double yn = __dmul_rn(ym1, y);
    const float rcp = __frcp_rn(__double2float_rn(__dmul_rn(static_cast<double>(N), ym1)));
    y = __dsub_rn(y, __dmul_rn(__dsub_rn(yn, z), static_cast<double>(rcp)));
  }
  y = rootn_fix<N>(z, y, 0.0);
  const double m = __longlong_as_double(
      static_cast<long long>((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull));
  const double u = __ddiv_rn(__dsub_rn(m, 1.0), __dadd_rn(m, 1.0));
  const double u2 = __dmul_rn(u, u);
  const double lnm = __dmul_rn(
      __dmul_rn(2.0, u),
      __dadd_rn(1.0, __dmul_rn(u2, __dadd_rn(1.0 / 3.0, __dmul_rn(u2, __dadd_rn(1.0 / 5.0, __dmul_rn(u2, 1.0 / 7.0)))))));
  const double lnx = __dadd_rn(__dmul_rn(static_cast<double>(e - shift), 0.6931471805599453), lnm);
  const double delta = (N == 3) ? -0x1p-54 / 3.0 : 0x1p-54 / 5.0;
  const double c = __dmul_rn(delta, lnx);
  y = __fma_rn(y, c, y);
  y = rootn_fix<N>(z, y, __dmul_rn(z, __dmul_rn(static_cast<double>(N), c)));
  return __dmul_rn(__dmul_rn(y, __longlong_as_double(static_cast<long long>(static_cast<unsigned long long>(1023 + q) << 52))), s);
}

}  // namespace bacon
