// RKF45 kernels, exact FP64 arithmetic, tableau variant 2.
#include "rk_inst.cuh"

namespace bacon {
void register_rk45_exact_l2(std::vector<RkEntry>& v) {
  register_rk_set<Rkf45Literal, 2, ExactOps>(v, 0, 0);
}
}  // namespace bacon
