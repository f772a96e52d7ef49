// Instantiation helper for the adjoint: recording forward kernel plus reverse
// kernel for every right-hand side that has a vector-Jacobian product.
#pragma once

#include "registry.h"
#include "rk_adjoint.cuh"

namespace bacon {

constexpr int kAdjMaxSegment = 32;

template <class Lit, int L>
void register_adjoint_set(std::vector<AdjEntry>& v, int method) {
  auto add = [&](auto tag, int rhs_id) {
    using R = typename decltype(tag)::type;
    using T = Tableau<Lit, L>;
    v.push_back(AdjEntry{RkKey{method, L, 0, rhs_id, R::DIM},
                         reinterpret_cast<const void*>(&rk_persistent_kernel<T, R, ExactOps, true>),
                         reinterpret_cast<const void*>(&rk_adjoint_reverse_kernel<T, R, kAdjMaxSegment>)});
  };
  add(TypeTag<RhsExp<1>>{}, kRhsExp);
  add(TypeTag<RhsExp<2>>{}, kRhsExp);
  add(TypeTag<RhsDecay<1>>{}, kRhsDecay);
  add(TypeTag<RhsDecay<2>>{}, kRhsDecay);
  add(TypeTag<RhsHarmonic>{}, kRhsHarmonic);
  add(TypeTag<RhsVdp>{}, kRhsVdp);
  add(TypeTag<RhsLorenz>{}, kRhsLorenz);
  add(TypeTag<RhsLotka>{}, kRhsLotka);
}

}  // namespace bacon
