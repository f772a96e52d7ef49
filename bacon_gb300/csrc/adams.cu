// Instantiations of the batched Adams (orders 5 and 3) and Euler kernels for
// the non-stiff right-hand sides of the registry.
#include "adams.h"
#include "adams_kernel.cuh"

namespace bacon {

namespace {
template <class R>
void add(std::vector<AdamsEntry>& v, int rhs_id) {
  v.push_back(AdamsEntry{5, rhs_id, R::DIM, reinterpret_cast<const void*>(&adams_persistent_kernel<5, R>)});
  v.push_back(AdamsEntry{3, rhs_id, R::DIM, reinterpret_cast<const void*>(&adams_persistent_kernel<3, R>)});
  v.push_back(AdamsEntry{1, rhs_id, R::DIM, reinterpret_cast<const void*>(&euler_persistent_kernel<R>)});
}
}  // namespace

std::vector<AdamsEntry> all_adams_kernels() {
  std::vector<AdamsEntry> v;
  add<RhsExp<1>>(v, kRhsExp);
  add<RhsExp<2>>(v, kRhsExp);
  add<RhsDecay<1>>(v, kRhsDecay);
  add<RhsDecay<2>>(v, kRhsDecay);
  add<RhsQuadratic<1>>(v, kRhsQuadratic);
  add<RhsSine<1>>(v, kRhsSine);
  add<RhsHarmonic>(v, kRhsHarmonic);
  add<RhsVdp>(v, kRhsVdp);
  add<RhsLorenz>(v, kRhsLorenz);
  add<RhsLotka>(v, kRhsLotka);
  return v;
}

}  // namespace bacon
