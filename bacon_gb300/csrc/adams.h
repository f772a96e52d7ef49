// Registry of the batched Adams and Euler kernels.
#pragma once

#include <vector>

namespace bacon {

struct AdamsEntry {
  int order;  // 5 (Adams5), 3 (Adams3), 1 (Euler)
  int rhs;
  int dim;
  const void* fn;  // __global__ void(AdamsArgs)
};

std::vector<AdamsEntry> all_adams_kernels();

}  // namespace bacon
