// Instantiation helper: registers one (tableau variant, arithmetic policy)
// kernel for every right-hand side of the registry that fits one thread.
#pragma once

#include "registry.h"
#include "rk_kernel.cuh"

namespace bacon {

template <class Lit, int L, class Ops>
void register_rk_set(std::vector<RkEntry>& v, int method, int prec) {
  auto add = [&](auto tag, int rhs_id) {
    using R = typename decltype(tag)::type;
    v.push_back(RkEntry{RkKey{method, L, prec, rhs_id, R::DIM},
                        reinterpret_cast<const void*>(&rk_persistent_kernel<Tableau<Lit, L>, R, Ops>)});
  };
  add(TypeTag<RhsExp<1>>{}, kRhsExp);
  add(TypeTag<RhsExp<2>>{}, kRhsExp);
  add(TypeTag<RhsDecay<1>>{}, kRhsDecay);
  add(TypeTag<RhsDecay<2>>{}, kRhsDecay);
  add(TypeTag<RhsQuadratic<1>>{}, kRhsQuadratic);
  add(TypeTag<RhsSine<1>>{}, kRhsSine);
  add(TypeTag<RhsSine<2>>{}, kRhsSine);
  add(TypeTag<RhsHarmonic>{}, kRhsHarmonic);
  add(TypeTag<RhsVdp>{}, kRhsVdp);
  add(TypeTag<RhsLorenz>{}, kRhsLorenz);
  add(TypeTag<RhsLotka>{}, kRhsLotka);
  add(TypeTag<RhsRobertson>{}, kRhsRobertson);
}

}  // namespace bacon
