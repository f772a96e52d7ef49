// Host/device interface of the plain one-launch-per-attempt baseline.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace bacon {

constexpr int32_t kPlainRunning = -1;

struct PlainArgs {
  int64_t n;
  int32_t stages;
  int32_t dim;
  double* y;          // [D][n]   current (last yielded) state
  double* K;          // [S][D][n] stage values, kept across attempts
  double* t;          // [n]
  double* dt;         // [n]
  double* end;        // [n]
  int64_t* attempts;  // [n]
  int32_t* accepted;  // [n]
  int32_t* rejected;  // [n]
  int32_t* status;    // [n]  kPlainRunning while integrating
  const double* params;  // [P][n]
  unsigned int* live;    // systems still running after this launch
  double tol, dt_min, dt_max;
  int64_t max_attempts;
};

struct PlainTables {
  int stages;
  double m[6][6];
  double c[6];
  double b[6];
  double e[6];
};

bool plain_tables(int method, int layout, PlainTables& tb);
cudaError_t plain_upload_tables(const PlainTables& tb, cudaStream_t s);
const void* plain_kernel(int rhs, int dim);
const void* plain_init_kernel();

struct PlainInitArgs {
  int64_t n;
  int32_t dim;
  int32_t stages;
  const double* y0;
  const double* t0;
  const double* t_end;
  double t0_s, t_end_s, dt0;
  PlainArgs st;
};

}  // namespace bacon
