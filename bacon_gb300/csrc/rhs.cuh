// Device right-hand sides of the engine's registry.
//
// The reference accepts any Rust closure f(t, y, &mut data) (src/ivp.rs:34-48);
// a GPU kernel cannot call host code, so the engine compiles a fixed set of
// right-hand sides.  Each expression is written with explicit evaluation
// order through the arithmetic policy `Ops`, so the exact-mode kernels and the
// CPU restatement evaluate the same rounded operations.  The first five are
// the right-hand sides of the reference's own tests (src/ivp/rk.rs:664-670,
// src/ivp/bdf.rs:769-783, src/ivp.rs:527-529).
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
  template <class Ops>
  __device__ __forceinline__ static void eval(double, const double (&y)[D], const double*, double (&f)[D]) {
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = y[d];
  }
};

template <int D>
struct RhsDecay {  // y' = -y
  static constexpr int DIM = D, NP = 0;
  static constexpr bool kUsesT = false;
  template <class Ops>
  __device__ __forceinline__ static void eval(double, const double (&y)[D], const double*, double (&f)[D]) {
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = -y[d];
  }
};

template <int D>
struct RhsQuadratic {  // y' = -2 t
  static constexpr int DIM = D, NP = 0;
  static constexpr bool kUsesT = true;
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
  template <class Ops>
  __device__ __forceinline__ static void eval(double, const double (&y)[2], const double*, double (&f)[2]) {
    f[0] = y[1];
    f[1] = -y[0];
  }
};

struct RhsVdp {  // y0' = y1, y1' = mu (1 - y0^2) y1 - y0
  static constexpr int DIM = 2, NP = 1;
  static constexpr bool kUsesT = false;
  template <class Ops>
  __device__ __forceinline__ static void eval(double, const double (&y)[2], const double* p, double (&f)[2]) {
    f[0] = y[1];
    f[1] = Ops::sub(Ops::mul(Ops::mul(p[0], Ops::sub(1.0, Ops::mul(y[0], y[0]))), y[1]), y[0]);
  }
};

struct RhsLorenz {  // sigma (y1 - y0), y0 (rho - y2) - y1, y0 y1 - beta y2
  static constexpr int DIM = 3, NP = 3;
  static constexpr bool kUsesT = false;
  template <class Ops>
  __device__ __forceinline__ static void eval(double, const double (&y)[3], const double* p, double (&f)[3]) {
    f[0] = Ops::mul(p[0], Ops::sub(y[1], y[0]));
    f[1] = Ops::sub(Ops::mul(y[0], Ops::sub(p[1], y[2])), y[1]);
    f[2] = Ops::sub(Ops::mul(y[0], y[1]), Ops::mul(p[2], y[2]));
  }
};

struct RhsLotka {  // a x - b x y, c x y - d y
  static constexpr int DIM = 2, NP = 4;
  static constexpr bool kUsesT = false;
  template <class Ops>
  __device__ __forceinline__ static void eval(double, const double (&y)[2], const double* p, double (&f)[2]) {
    f[0] = Ops::sub(Ops::mul(p[0], y[0]), Ops::mul(Ops::mul(p[1], y[0]), y[1]));
    f[1] = Ops::sub(Ops::mul(Ops::mul(p[2], y[0]), y[1]), Ops::mul(p[3], y[1]));
  }
};

struct RhsRobertson {  // k1, k2, k3 kinetics
  static constexpr int DIM = 3, NP = 3;
  static constexpr bool kUsesT = false;
  template <class Ops>
  __device__ __forceinline__ static void eval(double, const double (&y)[3], const double* p, double (&f)[3]) {
    const double r1 = Ops::mul(p[0], y[0]);
    const double r2 = Ops::mul(Ops::mul(p[1], y[1]), y[1]);
    const double r3 = Ops::mul(Ops::mul(p[2], y[1]), y[2]);
    f[0] = Ops::sub(r3, r1);
    f[1] = Ops::sub(Ops::sub(r1, r2), r3);
    f[2] = r2;
  }
};

}  // namespace bacon
