// Register-budget variants of the persistent Runge-Kutta kernels for the
// benchmark right-hand sides (Van der Pol, Lorenz-63, Lotka-Volterra) with the
// fehlberg reading of RKF45, exact FP64 and FP32-stage.  Variant 1 caps a
// thread at 80 registers (launch bounds 256 x 3), variant 2 at 64 (256 x 4);
// results are bit-identical to the default kernel's, only spills and
// occupancy differ.  bacon_rk_autotune times them on the caller's batch.
#include "registry.h"
#include "rk_ff_kernel.cuh"
#include "rk_kernel.cuh"

namespace bacon {

namespace {
template <int kMinBlocks, int kVariant>
void register_budget(std::vector<RkEntry>& v) {
  using T = Tableau<Rkf45Literal, kFehlberg>;
  auto add = [&](auto tag, int rhs_id) {
    using R = typename decltype(tag)::type;
    v.push_back(RkEntry{RkKey{0, kFehlberg, 0, rhs_id, R::DIM},
                        reinterpret_cast<const void*>(&rk_persistent_kernel<T, R, ExactOps, false, kMinBlocks>),
                        kVariant});
    v.push_back(RkEntry{RkKey{0, kFehlberg, 2, rhs_id, R::DIM},
                        reinterpret_cast<const void*>(&rk_persistent_ff_kernel<T, R, kMinBlocks>), kVariant});
  };
  add(TypeTag<RhsVdp>{}, kRhsVdp);
  add(TypeTag<RhsLorenz>{}, kRhsLorenz);
  add(TypeTag<RhsLotka>{}, kRhsLotka);
}
}  // namespace

void register_rk_variants(std::vector<RkEntry>& v) {
  register_budget<3, 1>(v);
  register_budget<4, 2>(v);
}

}  // namespace bacon
