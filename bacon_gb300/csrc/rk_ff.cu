// FP32-stage (float-float) kernels, every tableau reading, autonomous
// right-hand sides.
#include "registry.h"
#include "rk_ff_kernel.cuh"

namespace bacon {

namespace {
template <class Lit, int L>
void register_ff_set(std::vector<RkEntry>& v, int method) {
  auto add = [&](auto tag, int rhs_id) {
    using R = typename decltype(tag)::type;
    v.push_back(RkEntry{RkKey{method, L, 2, rhs_id, R::DIM},
                        reinterpret_cast<const void*>(&rk_persistent_ff_kernel<Tableau<Lit, L>, R>)});
  };
  add(TypeTag<RhsExp<1>>{}, kRhsExp);
  add(TypeTag<RhsExp<2>>{}, kRhsExp);
  add(TypeTag<RhsDecay<1>>{}, kRhsDecay);
  add(TypeTag<RhsDecay<2>>{}, kRhsDecay);
  add(TypeTag<RhsHarmonic>{}, kRhsHarmonic);
  add(TypeTag<RhsVdp>{}, kRhsVdp);
  add(TypeTag<RhsLorenz>{}, kRhsLorenz);
  add(TypeTag<RhsLotka>{}, kRhsLotka);
  add(TypeTag<RhsRobertson>{}, kRhsRobertson);
}
}  // namespace

void register_rk_ff(std::vector<RkEntry>& v) {
  register_ff_set<Rkf45Literal, kAsCompiled>(v, 0);
  register_ff_set<Rkf45Literal, kAsWritten>(v, 0);
  register_ff_set<Rkf45Literal, kFehlberg>(v, 0);
  register_ff_set<Bs23Literal, kAsCompiled>(v, 1);
  register_ff_set<Bs23Literal, kAsWritten>(v, 1);
}

}  // namespace bacon
