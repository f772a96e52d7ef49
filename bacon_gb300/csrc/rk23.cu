// Bogacki-Shampine 3(2) kernels (RungeKutta23), both readings of the matrix,
// exact and contracted arithmetic.  The fehlberg variant maps to as_written.
#include "rk_inst.cuh"

namespace bacon {
void register_rk23(std::vector<RkEntry>& v) {
  register_rk_set<Bs23Literal, kAsCompiled, ExactOps>(v, 1, 0);
  register_rk_set<Bs23Literal, kAsWritten, ExactOps>(v, 1, 0);
  register_rk_set<Bs23Literal, kAsCompiled, FmaOps>(v, 1, 1);
  register_rk_set<Bs23Literal, kAsWritten, FmaOps>(v, 1, 1);
}
}  // namespace bacon
