// Device right-hand sides of the engine's registry.
//
// The reference accepts any Rust closure f(t, y, &mut data) (src/ivp.rs:34-48);
// a GPU kernel cannot call host code, so the engine compiles a fixed set of
// right-hand sides.  Each expression is written with explicit evaluation
// order through the arithmetic policy `Ops`, so the exact-mode kernels and the
// CPU restatement evaluate the same rounded operations.  The first five are
// the right-hand sides of the reference's own tests (src/ivp/rk.rs:664-670,
// src/ivp/bdf.rs:769-783, src/ivp.rs:527-529).  kAffine marks the ones affine
// in y (f = J y + g(t) with J constant): with their exact Jacobian the
// corrected BDF's Newton solve ends after its first update.
#pragma once

#include "device_math.cuh"

namespace bacon {

enum RhsId : int {
  kRhsExp = 0,
  kRhsDecay = 1,
  kRhsQuadratic = 2,
  kRhsSine = 3,
  kRhsHarmonic = 4,
  kRhsVdp = 5,
  kRhsLorenz = 6,
  kRhsLotka = 7,
  kRhsRobertson = 8,
  kRhsChain = 9,
  kRhsLinear = 10,
};

template <int D>
struct RhsExp {  // y' = y
  static constexpr int DIM = D, NP = 0;
  static constexpr bool kUsesT = false;
  static constexpr bool kAffine = true;
  template <class Ops, class V>
  __device__ __forceinline__ static void eval(double, const V (&y)[D], const V*, V (&f)[D]) {
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = y[d];
  }
};

template <int D>
struct RhsDecay {  // y' = -y
  static constexpr int DIM = D, NP = 0;
  static constexpr bool kUsesT = false;
  static constexpr bool kAffine = true;
  template <class Ops, class V>
  __device__ __forceinline__ static void eval(double, const V (&y)[D], const V*, V (&f)[D]) {
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = -y[d];
  }
};

template <int D>
struct RhsQuadratic {  // y' = -2 t
  static constexpr int DIM = D, NP = 0;
  static constexpr bool kUsesT = true;
  static constexpr bool kAffine = true;
  template <class Ops>
  __device__ __forceinline__ static void eval(double t, const double (&)[D], const double*, double (&f)[D]) {
    const double v = Ops::mul(-2.0, t);
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = v;
  }
};

template <int D>
struct RhsSine {  // y' = cos t
  static constexpr int DIM = D, NP = 0;
  static constexpr bool kUsesT = true;
  static constexpr bool kAffine = true;
  template <class Ops>
  __device__ __forceinline__ static void eval(double t, const double (&)[D], const double*, double (&f)[D]) {
    const double v = cos(t);
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = v;
  }
};

struct RhsHarmonic {  // (y1, -y0)
  static constexpr int DIM = 2, NP = 0;
  static constexpr bool kUsesT = false;
  static constexpr bool kAffine = true;
  template <class Ops, class V>
  __device__ __forceinline__ static void eval(double, const V (&y)[2], const V*, V (&f)[2]) {
    f[0] = y[1];
    f[1] = -y[0];
  }
};

struct RhsVdp {  // y0' = y1, y1' = mu (1 - y0^2) y1 - y0
  static constexpr int DIM = 2, NP = 1;
  static constexpr bool kUsesT = false;
  static constexpr bool kAffine = false;
  template <class Ops, class V>
  __device__ __forceinline__ static void eval(double, const V (&y)[2], const V* p, V (&f)[2]) {
    f[0] = y[1];
    f[1] = Ops::sub(Ops::mul(Ops::mul(p[0], Ops::sub(1.0, Ops::mul(y[0], y[0]))), y[1]), y[0]);
  }
};

struct RhsLorenz {  // sigma (y1 - y0), y0 (rho - y2) - y1, y0 y1 - beta y2
  static constexpr int DIM = 3, NP = 3;
  static constexpr bool kUsesT = false;
  static constexpr bool kAffine = false;
  template <class Ops, class V>
  __device__ __forceinline__ static void eval(double, const V (&y)[3], const V* p, V (&f)[3]) {
    f[0] = Ops::mul(p[0], Ops::sub(y[1], y[0]));
    f[1] = Ops::sub(Ops::mul(y[0], Ops::sub(p[1], y[2])), y[1]);
    f[2] = Ops::sub(Ops::mul(y[0], y[1]), Ops::mul(p[2], y[2]));
  }
};

struct RhsLotka {  // a x - b x y, c x y - d y
  static constexpr int DIM = 2, NP = 4;
  static constexpr bool kUsesT = false;
  static constexpr bool kAffine = false;
  template <class Ops, class V>
  __device__ __forceinline__ static void eval(double, const V (&y)[2], const V* p, V (&f)[2]) {
    f[0] = Ops::sub(Ops::mul(p[0], y[0]), Ops::mul(Ops::mul(p[1], y[0]), y[1]));
    f[1] = Ops::sub(Ops::mul(Ops::mul(p[2], y[0]), y[1]), Ops::mul(p[3], y[1]));
  }
};

// Damped spring-mass chain, N masses: y = (x_0..x_{N-1}, v_0..v_{N-1}),
// spring i joins mass i-1 (a wall for i = 0) and mass i with stiffness p[i],
// damping p[N] on every (unit) mass.
template <int N>
struct RhsChain {
  static constexpr int DIM = 2 * N, NP = N + 1;
  static constexpr bool kUsesT = false;
  static constexpr bool kAffine = true;
  template <class Ops, class V>
  __device__ __forceinline__ static void eval(double, const V (&y)[2 * N], const V* p, V (&f)[2 * N]) {
    const V c = p[N];
#pragma unroll
    for (int i = 0; i < N; ++i) f[i] = y[N + i];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const V xl = (i == 0) ? V(0.0) : y[i - 1];
      const V xr = (i + 1 < N) ? y[i + 1] : V(0.0);
      const V kl = p[i];
      const V kr = (i + 1 < N) ? p[i + 1] : V(0.0);
      const V force = Ops::add(Ops::mul(kl, Ops::sub(xl, y[i])), Ops::mul(kr, Ops::sub(xr, y[i])));
      f[N + i] = Ops::sub(force, Ops::mul(c, y[N + i]));
    }
  }
};

// ---- Jacobians for the implicit (BDF) solvers ------------------------------
// J[r][c] = d f_r / d y_c, the same expressions and order as the CPU oracle's
// oracle_rhs_jacobian.
template <class R>
struct Jac;

template <int D>
struct Jac<RhsExp<D>> {
  template <class Ops>
  __device__ __forceinline__ static void eval(const double (&)[D], const double*, double (&J)[D][D]) {
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int c = 0; c < D; ++c) J[r][c] = (r == c) ? 1.0 : 0.0;
  }
};

template <int D>
struct Jac<RhsDecay<D>> {
  template <class Ops>
  __device__ __forceinline__ static void eval(const double (&)[D], const double*, double (&J)[D][D]) {
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int c = 0; c < D; ++c) J[r][c] = (r == c) ? -1.0 : 0.0;
  }
};

template <int D>
struct Jac<RhsQuadratic<D>> {
  template <class Ops>
  __device__ __forceinline__ static void eval(const double (&)[D], const double*, double (&J)[D][D]) {
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int c = 0; c < D; ++c) J[r][c] = 0.0;
  }
};

template <int D>
struct Jac<RhsSine<D>> {
  template <class Ops>
  __device__ __forceinline__ static void eval(const double (&)[D], const double*, double (&J)[D][D]) {
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int c = 0; c < D; ++c) J[r][c] = 0.0;
  }
};

template <>
struct Jac<RhsVdp> {
  template <class Ops>
  __device__ __forceinline__ static void eval(const double (&y)[2], const double* p, double (&J)[2][2]) {
    const double mu = p[0];
    J[0][0] = 0.0;
    J[0][1] = 1.0;
    J[1][0] = Ops::sub(Ops::mul(Ops::mul(Ops::mul(-2.0, mu), y[0]), y[1]), 1.0);
    J[1][1] = Ops::mul(mu, Ops::sub(1.0, Ops::mul(y[0], y[0])));
  }
};

template <>
struct Jac<RhsLorenz> {
  template <class Ops>
  __device__ __forceinline__ static void eval(const double (&y)[3], const double* p, double (&J)[3][3]) {
    J[0][0] = -p[0];
    J[0][1] = p[0];
    J[0][2] = 0.0;
    J[1][0] = Ops::sub(p[1], y[2]);
    J[1][1] = -1.0;
    J[1][2] = -y[0];
    J[2][0] = y[1];
    J[2][1] = y[0];
    J[2][2] = -p[2];
  }
};

template <>
struct Jac<RhsLotka> {
  template <class Ops>
  __device__ __forceinline__ static void eval(const double (&y)[2], const double* p, double (&J)[2][2]) {
    J[0][0] = Ops::sub(p[0], Ops::mul(p[1], y[1]));
    J[0][1] = -Ops::mul(p[1], y[0]);
    J[1][0] = Ops::mul(p[2], y[1]);
    J[1][1] = Ops::sub(Ops::mul(p[2], y[0]), p[3]);
  }
};

template <int N>
struct Jac<RhsChain<N>> {
  template <class Ops>
  __device__ __forceinline__ static void eval(const double (&)[2 * N], const double* p,
                                              double (&J)[2 * N][2 * N]) {
    constexpr int D = 2 * N;
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int c = 0; c < D; ++c) J[r][c] = 0.0;
    const double c = p[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      J[i][N + i] = 1.0;
      const double kl = p[i];
      const double kr = (i + 1 < N) ? p[i + 1] : 0.0;
      J[N + i][i] = -Ops::add(kl, kr);
      if (i > 0) J[N + i][i - 1] = kl;
      if (i + 1 < N) J[N + i][i + 1] = kr;
      J[N + i][N + i] = -c;
    }
  }
};

// ---- vector-Jacobian products for the discrete adjoint --------------------
// ubar = J_f(y)^T v, and mu += (df/dp)(y)^T v.  The reference has no
// gradients; this is the adjoint's own arithmetic, with fused multiply-adds
// (one rounding each) in the same order as the CPU oracle's rhs_vjp
// (oracle/adjoint_oracle.c), so that the adjoint is bit-reproducible.
template <class R>
struct Vjp;

template <int D>
struct Vjp<RhsExp<D>> {
  __device__ __forceinline__ static void eval(const double (&)[D], const double*, const double (&v)[D],
                                              double (&ub)[D], double*) {
#pragma unroll
    for (int d = 0; d < D; ++d) ub[d] = v[d];
  }
};

template <int D>
struct Vjp<RhsDecay<D>> {
  __device__ __forceinline__ static void eval(const double (&)[D], const double*, const double (&v)[D],
                                              double (&ub)[D], double*) {
#pragma unroll
    for (int d = 0; d < D; ++d) ub[d] = -v[d];
  }
};

template <>
struct Vjp<RhsHarmonic> {
  __device__ __forceinline__ static void eval(const double (&)[2], const double*, const double (&v)[2],
                                              double (&ub)[2], double*) {
    ub[0] = -v[1];
    ub[1] = v[0];
  }
};

template <>
struct Vjp<RhsVdp> {
  __device__ __forceinline__ static void eval(const double (&y)[2], const double* p, const double (&v)[2],
                                              double (&ub)[2], double* mu) {
    const double m = p[0];
    const double w = __fma_rn(-y[0], y[0], 1.0);
    ub[0] = __dmul_rn(__fma_rn(__dmul_rn(__dmul_rn(-2.0, m), y[0]), y[1], -1.0), v[1]);
    ub[1] = __fma_rn(__dmul_rn(m, w), v[1], v[0]);
    mu[0] = __fma_rn(__dmul_rn(w, y[1]), v[1], mu[0]);
  }
};

template <>
struct Vjp<RhsLorenz> {
  __device__ __forceinline__ static void eval(const double (&y)[3], const double* p, const double (&v)[3],
                                              double (&ub)[3], double* mu) {
    const double s = p[0], r = p[1], b = p[2];
    ub[0] = __fma_rn(y[1], v[2], __fma_rn(__dsub_rn(r, y[2]), v[1], __dmul_rn(-s, v[0])));
    ub[1] = __fma_rn(y[0], v[2], __fma_rn(s, v[0], -v[1]));
    ub[2] = __fma_rn(-y[0], v[1], -__dmul_rn(b, v[2]));
    mu[0] = __fma_rn(__dsub_rn(y[1], y[0]), v[0], mu[0]);
    mu[1] = __fma_rn(y[0], v[1], mu[1]);
    mu[2] = __fma_rn(-y[2], v[2], mu[2]);
  }
};

template <>
struct Vjp<RhsLotka> {
  __device__ __forceinline__ static void eval(const double (&y)[2], const double* p, const double (&v)[2],
                                              double (&ub)[2], double* mu) {
    const double a = p[0], b = p[1], c = p[2], dd = p[3];
    const double x = y[0], w = y[1];
    ub[0] = __fma_rn(__dmul_rn(c, w), v[1], __dmul_rn(__fma_rn(-b, w, a), v[0]));
    ub[1] = __fma_rn(__fma_rn(c, x, -dd), v[1], __dmul_rn(-__dmul_rn(b, x), v[0]));
    const double xw = __dmul_rn(x, w);
    mu[0] = __fma_rn(x, v[0], mu[0]);
    mu[1] = __fma_rn(-xw, v[0], mu[1]);
    mu[2] = __fma_rn(xw, v[1], mu[2]);
    mu[3] = __fma_rn(-w, v[1], mu[3]);
  }
};

struct RhsRobertson {  // k1, k2, k3 kinetics
  static constexpr int DIM = 3, NP = 3;
  static constexpr bool kUsesT = false;
  static constexpr bool kAffine = false;
  template <class Ops, class V>
  __device__ __forceinline__ static void eval(double, const V (&y)[3], const V* p, V (&f)[3]) {
    const V r1 = Ops::mul(p[0], y[0]);
    const V r2 = Ops::mul(Ops::mul(p[1], y[1]), y[1]);
    const V r3 = Ops::mul(Ops::mul(p[2], y[1]), y[2]);
    f[0] = Ops::sub(r3, r1);
    f[1] = Ops::sub(Ops::sub(r1, r2), r3);
    f[2] = r2;
  }
};

template <>
struct Jac<RhsRobertson> {
  template <class Ops>
  __device__ __forceinline__ static void eval(const double (&y)[3], const double* p, double (&J)[3][3]) {
    const double k1 = p[0], k2 = p[1], k3 = p[2];
    J[0][0] = -k1;
    J[0][1] = Ops::mul(k3, y[2]);
    J[0][2] = Ops::mul(k3, y[1]);
    J[1][0] = k1;
    J[1][1] = Ops::sub(Ops::mul(Ops::mul(-2.0, k2), y[1]), Ops::mul(k3, y[2]));
    J[1][2] = -Ops::mul(k3, y[1]);
    J[2][0] = 0.0;
    J[2][1] = Ops::mul(Ops::mul(2.0, k2), y[1]);
    J[2][2] = 0.0;
  }
};

template <>
struct Jac<RhsHarmonic> {
  template <class Ops>
  __device__ __forceinline__ static void eval(const double (&)[2], const double*, double (&J)[2][2]) {
    J[0][0] = 0.0;
    J[0][1] = 1.0;
    J[1][0] = -1.0;
    J[1][1] = 0.0;
  }
};

}  // namespace bacon
