// Kernel registry: every compiled (method, layout, precision, rhs, dim)
// combination of the persistent Runge-Kutta kernel, looked up at solve time.
#pragma once

#include <cstdint>
#include <vector>

namespace bacon {

struct RkKey {
  int method;     // 0 RK45, 1 RK23
  int layout;     // 0 as_compiled, 1 as_written, 2 fehlberg
  int precision;  // 0 fp64 exact, 1 fp64 fma, 2 fp32 compensated
  int rhs;
  int dim;
  bool operator==(const RkKey& o) const {
    return method == o.method && layout == o.layout && precision == o.precision && rhs == o.rhs &&
           dim == o.dim;
  }
};

struct RkEntry {
  RkKey key;
  const void* fn;   // __global__ void(RkArgs)
  int variant = 0;  // 0: the default kernel; >0: an autotuner alternative
};

// The autotuner's kernel variants of one key: a register budget set through
// the launch bounds (max_registers, 0 = the compiler's choice).
struct RkVariantInfo {
  int variant;
  int max_registers;
};

struct AdjEntry {
  RkKey key;
  const void* fwd;  // recording forward kernel, __global__ void(RkArgs)
  const void* rev;  // reverse kernel, __global__ void(AdjArgs)
};

template <class T>
struct TypeTag {
  using type = T;
};

void register_rk45_exact_l0(std::vector<RkEntry>& v);
void register_rk45_exact_l1(std::vector<RkEntry>& v);
void register_rk45_exact_l2(std::vector<RkEntry>& v);
void register_rk45_fma(std::vector<RkEntry>& v);
void register_rk23(std::vector<RkEntry>& v);
void register_rk_ff(std::vector<RkEntry>& v);
void register_rk_variants(std::vector<RkEntry>& v);
// Register budget of a variant id (variant 1: 80, 2: 64; 0: none).
inline int variant_max_registers(int variant) { return variant == 1 ? 80 : variant == 2 ? 64 : 0; }

// Threads per block of a persistent one-system-per-thread launch: `full`,
// halved (down to one warp) while half of it still holds a whole SM's share
// of the batch.  A batch too small to fill the GPU then spreads its warps over
// every SM instead of packing them onto a few: 4,096 systems in blocks of 128
// ran on 32 of the 152 SMs, where the FP64 pipe serialises their warps.
inline int default_block(int64_t n, int num_sms, int full) {
  const int64_t per_sm = (n + num_sms - 1) / num_sms;
  int block = full;
  while (block > 32 && block / 2 >= per_sm) block /= 2;
  return block;
}
void register_adjoint_rk45(std::vector<AdjEntry>& v);
void register_adjoint_rk23(std::vector<AdjEntry>& v);

inline std::vector<RkEntry> all_rk_kernels() {
  std::vector<RkEntry> v;
  register_rk45_exact_l0(v);
  register_rk45_exact_l1(v);
  register_rk45_exact_l2(v);
  register_rk45_fma(v);
  register_rk23(v);
  register_rk_ff(v);
  register_rk_variants(v);
  return v;
}

inline std::vector<AdjEntry> all_adjoint_kernels() {
  std::vector<AdjEntry> v;
  register_adjoint_rk45(v);
  register_adjoint_rk23(v);
  return v;
}

}  // namespace bacon
