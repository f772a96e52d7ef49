/* A plain C caller of the engine's C ABI (include/bacon_gb300.h), as the
 * Rust crate's FFI or any other foreign caller would bind it: a builder for
 * the solver options, a batch of Van der Pol systems in host memory, one
 * bacon_rk_solve, and the results written to a file for the test to compare.
 *
 *   solve_vdp OUT_FILE   (writes n, y_final[2][n], t_final[n], accepted[n],
 *                         rejected[n], status[n], the return code)
 */
#include <stdio.h>
#include <stdlib.h>

#include "bacon_gb300.h"

#define N 2048

static double y0[2 * N], mu[N], y_final[2 * N], t_final[N];
static int32_t accepted[N], rejected[N], status[N];

int main(int argc, char** argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: solve_vdp OUT_FILE\n");
    return 2;
  }
  /* deterministic inputs, mirrored by the test: y0 in [-2, 2]^2, mu in [0.1, 2] */
  for (int i = 0; i < N; ++i) {
    y0[i] = -2.0 + 4.0 * (double)((i * 37) % 101) / 100.0;
    y0[N + i] = -2.0 + 4.0 * (double)((i * 53) % 103) / 102.0;
    mu[i] = 0.1 + 1.9 * (double)((i * 29) % 97) / 96.0;
  }
  /* the problem through the builder, as the reference's IVPSolver chain */
  bacon_builder* b = NULL;
  bacon_problem p;
  int rc = bacon_builder_new(BACON_RK45, 2, &b);
  if (rc == BACON_OK) rc = bacon_builder_with_tolerance(b, 1e-6);
  if (rc == BACON_OK) rc = bacon_builder_with_minimum_dt(b, 1e-6);
  if (rc == BACON_OK) rc = bacon_builder_with_maximum_dt(b, 0.1);
  if (rc == BACON_OK) rc = bacon_builder_with_initial_time(b, 0.0);
  if (rc == BACON_OK) rc = bacon_builder_with_ending_time(b, 10.0);
  if (rc == BACON_OK) rc = bacon_builder_with_initial_conditions(b, y0, N);
  if (rc == BACON_OK) rc = bacon_builder_with_derivative(b, BACON_RHS_VDP, mu, 1);
  if (rc == BACON_OK) rc = bacon_builder_problem(b, &p);
  if (rc != BACON_OK) {
    fprintf(stderr, "builder: %d %s\n", rc, bacon_last_error());
    bacon_builder_free(b);
    return 1;
  }
  bacon_ctx* ctx = NULL;
  if ((rc = bacon_ctx_create(0, &ctx)) != BACON_OK) {
    fprintf(stderr, "context: %d %s\n", rc, bacon_last_error());
    bacon_builder_free(b);
    return 1;
  }
  bacon_rk_options o = {0};
  o.method = BACON_RK45;
  o.layout = BACON_LAYOUT_FEHLBERG;
  o.precision = BACON_FP64_EXACT;
  o.memory = BACON_MEM_HOST;
  o.use_graph = 1;
  bacon_rk_result r = {0};
  r.y_final = y_final;
  r.t_final = t_final;
  r.accepted = accepted;
  r.rejected = rejected;
  r.status = status;
  const int solve_rc = bacon_rk_solve(ctx, &p, &o, &r);
  bacon_ctx_destroy(ctx);
  bacon_builder_free(b);

  FILE* f = fopen(argv[1], "wb");
  if (!f) return 1;
  const int64_t n = N;
  int ok = fwrite(&n, sizeof n, 1, f) == 1 && fwrite(y_final, sizeof(double), 2 * N, f) == 2 * N &&
           fwrite(t_final, sizeof(double), N, f) == N && fwrite(accepted, sizeof(int32_t), N, f) == N &&
           fwrite(rejected, sizeof(int32_t), N, f) == N && fwrite(status, sizeof(int32_t), N, f) == N &&
           fwrite(&solve_rc, sizeof solve_rc, 1, f) == 1;
  fclose(f);
  return ok ? 0 : 1;
}
