// Instantiations of the mixed stiff-batch kernel (ragged chains, one warp
// each, plus an optional uniform batch of small systems, one thread each).
#include "bdf.h"
#include "bdf_ragged.cuh"

namespace bacon {

const void* bdf_mixed_kernel_for(int small_rhs, int small_dim) {
  if (small_rhs < 0) return reinterpret_cast<const void*>(&bdf_mixed_kernel<NoSmall>);
  if (small_rhs == kRhsRobertson && small_dim == 3) return reinterpret_cast<const void*>(&bdf_mixed_kernel<RhsRobertson>);
  if (small_rhs == kRhsVdp && small_dim == 2) return reinterpret_cast<const void*>(&bdf_mixed_kernel<RhsVdp>);
  return nullptr;
}

}  // namespace bacon
