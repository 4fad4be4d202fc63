/*
 * qdeq_functions.h -- drop-in C++ surface: the reference's hot-path
 * functions (functions.h:11-45) with their signatures, over the C ABI of
 * qdeq.h.  Code that calls QDEqCycle_FDM's RK43 / setBoundary / NRsearch /
 * eval_stress_on_fault / cal_dpsi / computeError / computeStepSize /
 * extend_crew / SetMedium links against libqdeq_gb300.so instead.
 *
 * Differences a caller sees:
 *   - RK43 runs the whole adaptive loop on the GPU; it prints the reference's
 *     per-step line (odeSolver.cpp:1440,1636) and writes the reference's
 *     snapshot records (output_fault_<n>.bin, :1442-1457,1638-1652) into the
 *     directory set by qd_dropin_configure (default "output"), and on return
 *     leaves the final state in the caller's arrays;
 *   - errors are reported on stderr and end RK43 instead of exit();
 *   - SetMedium homogenises the caller's medium.mu (the reference also
 *     builds a hard-coded basin model there and dumps files);
 *   - ode_solve takes the solver in place of the reference's five device
 *     buffers and cuBLAS handle.
 */
#ifndef QDEQ_FUNCTIONS_H
#define QDEQ_FUNCTIONS_H

#include "qdeq.h"
#include "qdeq_struct.h"

#ifdef __cplusplus
extern "C" {
#endif
/* Multigrid schedule, prestress (NULL: none, as the reference), snapshot
 * directory and the tag printed at the head of each step line, for the
 * drop-in RK43.  Any argument may be NULL to keep its current value.
 * Defaults: qd_default_options(), no prestress, "output", "qdeq". */
void qd_dropin_configure(const qd_mg_options *opt, const double *tau0, const char *outdir,
                         const char *tag);
/* The solver the single-call drop-ins (eval_stress_on_fault, NRsearch,
 * cal_dpsi, ode_solve with a NULL solver) run on. */
void qd_dropin_bind(qd_solver *s);
#ifdef __cplusplus
}

void RK43(int method, GRID *grid, PARAMS *params, DISPLACEMENT U, FAULT fault, MEDIUM medium,
          RATE_STATE_LAW RSL);
void ode_solve(int method, GRID *grid, DISPLACEMENT U, qd_solver *solver);
void extend_crew(GRID *grid, DISPLACEMENT U);
void setBoundary(GRID *grid, DISPLACEMENT U, FAULT fault, RATE_STATE_LAW RSL, VARIABLE y,
                 PARAMS *params, double ratio);
void eval_stress_on_fault(GRID *grid, DISPLACEMENT U, PARAMS *params, FAULT fault, MEDIUM medium);
void NRsearch(GRID *grid, FAULT fault, RATE_STATE_LAW RSL, VARIABLE y, Runge_Kutta rk4);
void cal_dpsi(GRID *grid, RATE_STATE_LAW RSL, FAULT fault, VARIABLE y, Runge_Kutta rk4);
double computeError(GRID *grid, VARIABLE y3, VARIABLE y4);
double computeStepSize(GRID *grid, PARAMS *params, const double totErr, double totTol,
                       double errA[2]);
void SetMedium(GRID grid, COORD coord, MEDIUM medium, STRUCTURE structure);
#endif

#endif /* QDEQ_FUNCTIONS_H */
