// Discrete-adjoint kernels for Bogacki-Shampine 3(2).
#include "rk_adjoint_inst.cuh"

namespace bacon {
void register_adjoint_rk23(std::vector<AdjEntry>& v) { register_adjoint_set<Bs23Literal, kAsWritten>(v, 1); }
}  // namespace bacon
