// Right-hand sides compiled outside the engine, as a user of
// bacon_rk_solve_user writes them (include/bacon_gb300_rhs.cuh).
//
// UserVanDerPol repeats the registry's Van der Pol operation for operation,
// so its solve must be bit-identical to BACON_RHS_VDP.  UserDuffing is a
// system the registry does not have: the forced, damped Duffing oscillator
//   y0' = y1,  y1' = gamma cos(omega t) - delta y1 - alpha y0 - beta y0^3.
#include "bacon_gb300_rhs.cuh"

struct UserVanDerPol {
  static constexpr int DIM = 2, NP = 1;
  static constexpr bool kUsesT = false;
  template <class Ops, class V>
  __device__ __forceinline__ static void eval(double, const V (&y)[2], const V* p, V (&f)[2]) {
    f[0] = y[1];
    f[1] = Ops::sub(Ops::mul(Ops::mul(p[0], Ops::sub(1.0, Ops::mul(y[0], y[0]))), y[1]), y[0]);
  }
};

struct UserDuffing {  // p = (delta, alpha, beta, gamma, omega)
  static constexpr int DIM = 2, NP = 5;
  static constexpr bool kUsesT = true;
  template <class Ops, class V>
  __device__ __forceinline__ static void eval(double t, const V (&y)[2], const V* p, V (&f)[2]) {
    const double force = Ops::mul(p[3], cos(Ops::mul(p[4], t)));
    const double cubic = Ops::mul(p[2], Ops::mul(y[0], Ops::mul(y[0], y[0])));
    f[0] = y[1];
    f[1] = Ops::sub(Ops::sub(Ops::sub(force, Ops::mul(p[0], y[1])), Ops::mul(p[1], y[0])), cubic);
  }
};

BACON_DEFINE_RK_LAUNCHER(user_vdp_launch, UserVanDerPol)
BACON_DEFINE_RK_LAUNCHER(user_duffing_launch, UserDuffing)
