// Discrete-adjoint kernels for RKF45 (as_written and fehlberg readings).
#include "rk_adjoint_inst.cuh"

namespace bacon {
void register_adjoint_rk45(std::vector<AdjEntry>& v) {
  register_adjoint_set<Rkf45Literal, kAsWritten>(v, 0);
  register_adjoint_set<Rkf45Literal, kFehlberg>(v, 0);
}
}  // namespace bacon
