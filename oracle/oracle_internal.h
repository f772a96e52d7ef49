/* CPU ORACLE — TEST INFRASTRUCTURE ONLY.  Internal declarations shared by
 * the oracle's translation units. */
#ifndef BACON_ORACLE_INTERNAL_H
#define BACON_ORACLE_INTERNAL_H

#define ORC_MAX_STAGES 6
#define ORC_MAX_DIM 512
#define ORC_MAX_BDF_DIM 128

typedef struct {
  int s;
  double c[ORC_MAX_STAGES];
  double m[ORC_MAX_STAGES][ORC_MAX_STAGES]; /* matrix as read by row_iter */
  double b[ORC_MAX_STAGES];
  double e[ORC_MAX_STAGES];
} orc_tableau;

/* Tableau of the reference (src/ivp/rk.rs:435-525, :568-620) in the chosen
 * reading (ORC_LAYOUT_*). */
void orc_tableau_build(int method, int layout, orc_tableau* tb);

#include <stdint.h>
#include "oracle.h"

/* oracle_rk_solve_one with a log of every yielded step: the dt it used, its
 * start time and start state (y_log row-major [k][dim]), first log_cap. */
int32_t orc_rk_solve_core(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                          const double* p, const double* shared, double t0, double t_end,
                          const double* y0, double* y_out, double* t_out, int64_t* accepted,
                          int64_t* rejected, double* traj_t, double* traj_y, int64_t traj_cap,
                          double* dt_log, double* t_log, double* y_log, int64_t log_cap);

#endif
