// Float-float ("double-single") arithmetic on the FP32 pipe.
//
// A value is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits.  GB300 issues 128 FP32 lanes per clock per SM
// and only 2 FP64 lanes, so a Runge-Kutta stage evaluated in float-float
// costs a fraction of the FP64 version while keeping the stage values far
// more accurate than any tolerance the controller uses.
//
// Built from the published error-free transformations: Knuth's TwoSum,
// Dekker's FastTwoSum and the FMA-based TwoProduct.  Every operation is an
// explicit round-to-nearest intrinsic (__fadd_rn, __fmul_rn, __fmaf_rn), so
// no contraction can break the compensation terms.
#pragma once

namespace bacon {

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_make(float hi, float lo) { return ff{hi, lo}; }

// Exact split of a double into hi + lo (the FP64 subtraction is exact).
__device__ __forceinline__ ff ff_from_double(double x) {
  const float h = __double2float_rn(x);
  const float l = __double2float_rn(__dsub_rn(x, static_cast<double>(h)));
  return ff{h, l};
}

__device__ __forceinline__ double ff_to_double(ff a) {
  return __dadd_rn(static_cast<double>(a.hi), static_cast<double>(a.lo));
}

// Compile-time split of a constant (folded by the compiler).
__host__ __device__ constexpr ff ff_const(double x) {
  return ff{static_cast<float>(x), static_cast<float>(x - static_cast<double>(static_cast<float>(x)))};
}

// s + e == a + b exactly (Knuth).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// s + e == a + b exactly when |a| >= |b| (Dekker).
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  float h, l;
  fast_two_sum(s, e, h, l);
  return ff{h, l};
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }

__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  float h, l;
  fast_two_sum(p, e, h, l);
  return ff{h, l};
}

// a * c for a constant c that is exactly a float.
__device__ __forceinline__ ff ff_mul_f(ff a, float c) {
  const float p = __fmul_rn(a.hi, c);
  float e = __fmaf_rn(a.hi, c, -p);
  e = __fmaf_rn(a.lo, c, e);
  float h, l;
  fast_two_sum(p, e, h, l);
  return ff{h, l};
}

// s + a * c in one pass: the exact product of the high parts (FMA
// TwoProduct), one TwoSum with s.hi, the low-order terms folded in with FMAs,
// one FastTwoSum.  15 FP32 operations where ff_add(s, ff_mul(a, c)) takes 18;
// the low-order error stays at the level of ff_mul's.
__device__ __forceinline__ ff ff_mad(ff s, ff a, ff c) {
  const float p = __fmul_rn(a.hi, c.hi);
  const float pe = __fmaf_rn(a.hi, c.hi, -p);
  float t, te;
  two_sum(s.hi, p, t, te);
  float lo = __fadd_rn(te, __fadd_rn(s.lo, pe));
  lo = __fmaf_rn(a.hi, c.lo, lo);
  lo = __fmaf_rn(a.lo, c.hi, lo);
  float h, l;
  fast_two_sum(t, lo, h, l);
  return ff{h, l};
}

// s + a * c for a constant c that is exactly a float: 14 operations.
__device__ __forceinline__ ff ff_mad_f(ff s, ff a, float c) {
  const float p = __fmul_rn(a.hi, c);
  const float pe = __fmaf_rn(a.hi, c, -p);
  float t, te;
  two_sum(s.hi, p, t, te);
  float lo = __fadd_rn(te, __fadd_rn(s.lo, pe));
  lo = __fmaf_rn(a.lo, c, lo);
  float h, l;
  fast_two_sum(t, lo, h, l);
  return ff{h, l};
}

// Arithmetic policy with the same names as ExactOps / FmaOps, on ff values.
struct FfOps {
  static constexpr bool kExact = false;
  __device__ __forceinline__ static ff mul(ff a, ff b) { return ff_mul(a, b); }
  __device__ __forceinline__ static ff add(ff a, ff b) { return ff_add(a, b); }
  __device__ __forceinline__ static ff sub(ff a, ff b) { return ff_sub(a, b); }
  __device__ __forceinline__ static ff mul(double a, ff b) { return ff_mul(ff_const(a), b); }
  __device__ __forceinline__ static ff sub(double a, ff b) { return ff_sub(ff_const(a), b); }
  __device__ __forceinline__ static ff add(ff a, double b) { return ff_add(a, ff_const(b)); }
};

__device__ __forceinline__ ff operator-(ff a) { return ff_neg(a); }

}  // namespace bacon
