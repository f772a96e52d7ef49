// Batched BDF kernels, corrected (the engine's stiff BDF) mode, for systems
// small enough to live in one thread's registers and local memory (dim <= 8).
#include "bdf.h"
#include "bdf_kernel.cuh"

namespace bacon {

namespace {
template <class R>
void add(std::vector<BdfEntry>& v, int rhs_id) {
  v.push_back(BdfEntry{1, 0, rhs_id, R::DIM, reinterpret_cast<const void*>(&bdf_corrected_kernel<R>)});
}
}  // namespace

void register_bdf_corrected(std::vector<BdfEntry>& v) {
  add<RhsExp<1>>(v, kRhsExp);
  add<RhsDecay<1>>(v, kRhsDecay);
  add<RhsQuadratic<1>>(v, kRhsQuadratic);
  add<RhsSine<1>>(v, kRhsSine);
  add<RhsHarmonic>(v, kRhsHarmonic);
  add<RhsVdp>(v, kRhsVdp);
  add<RhsLorenz>(v, kRhsLorenz);
  add<RhsLotka>(v, kRhsLotka);
  add<RhsRobertson>(v, kRhsRobertson);
  add<RhsChain<2>>(v, kRhsChain);
  add<RhsChain<3>>(v, kRhsChain);
  add<RhsChain<4>>(v, kRhsChain);
}

}  // namespace bacon
