// Registry of the batched BDF kernels.
#pragma once

#include <vector>

namespace bacon {

struct BdfEntry {
  int mode;    // 0 as_compiled, 1 corrected
  int method;  // 0 BDF6, 1 BDF2 (corrected kernels take the order at run time: method 0)
  int rhs;
  int dim;
  const void* fn;  // __global__ void(BdfArgs, int dyn_dim)
};

void register_bdf_corrected(std::vector<BdfEntry>& v);

// Mixed stiff-batch kernel __global__ void(BdfArgs, int small_dyn, RaggedArgs)
// for a uniform part of (small_rhs, small_dim), or for none (small_rhs < 0);
// null when not compiled.
const void* bdf_mixed_kernel_for(int small_rhs, int small_dim);
void register_bdf_as_compiled(std::vector<BdfEntry>& v);

inline std::vector<BdfEntry> all_bdf_kernels() {
  std::vector<BdfEntry> v;
  register_bdf_corrected(v);
  register_bdf_as_compiled(v);
  return v;
}

}  // namespace bacon
