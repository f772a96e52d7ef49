// RKF45 kernels with fused multiply-add contraction, all tableau variants.
#include "rk_inst.cuh"

namespace bacon {
void register_rk45_fma(std::vector<RkEntry>& v) {
  register_rk_set<Rkf45Literal, kAsCompiled, FmaOps>(v, 0, 1);
  register_rk_set<Rkf45Literal, kAsWritten, FmaOps>(v, 0, 1);
  register_rk_set<Rkf45Literal, kFehlberg, FmaOps>(v, 0, 1);
}
}  // namespace bacon
