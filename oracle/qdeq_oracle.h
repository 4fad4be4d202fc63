/*
 * qdeq_oracle.h -- CPU restatement of the reference's per-stage hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * GB300 kernels and the timed CPU baseline ("port").  Only tests/,
 * __graft_entry__.smoke() and bench.py (its cpu_baseline leg and its
 * --impl reference arm) may load it.  The product library never links it.
 *
 * Every function follows the reference line by line (plain C, no FMA
 * contraction: built with -ffp-contract=off) and cites the file:line of
 * QDEqCycle_FDM it restates.  Arrays use the reference's layouts:
 *   - ghosted fields U, mu_node: nx*nz doubles, index i + k*nx
 *     (nx = ni + 2, nz = nk + 2; struct.h:49-72, odeSolver.cpp:24-38);
 *   - compact multigrid fields: N*K doubles, index k + j*K
 *     (N = nk rows along the fault, K = ni columns; odeSolver.cpp:669-677);
 *   - mu_equi: the staggered (2nx-1)*(2nz-1) array (odeSolver.cpp:337-589);
 *   - fault vectors: nz doubles, valid entries nk1-1 .. nk2-1 = 1 .. nk.
 */
#ifndef QDEQ_ORACLE_H
#define QDEQ_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define QO_MAXLEV 16

/* ---------------- multigrid (odeSolver.cpp:652-1147) ---------------- */
typedef struct qo_mg {
    int n_levels;           /* odeSolver.cpp:3 (6 in the reference)          */
    int nu_pre, nu_post;    /* sweeps of smooth() before/after recursion      */
    int nu_coarse;          /* sweeps of smooth() on the coarsest level       */
    int N[QO_MAXLEV], K[QO_MAXLEV], fc[QO_MAXLEV];
    double DH[QO_MAXLEV];
    int nx;                 /* K0 + 2*LEND: half-grid width is 2*nx-1         */
    const double *mu;       /* mu_equi (borrowed)                             */
    const double *mux, *muz;  /* the moduli the x- and z-faces read: mu, or
                               mu J and mu / J on a stretched grid          */
    double *own_x, *own_z;  /* their storage when a metric is set            */
    double *res[QO_MAXLEV], *res2[QO_MAXLEV], *err2[QO_MAXLEV];
    double *delta;          /* level-0 residual buffer (delta_res)            */
    double *rowsum;         /* per-row partial sums for a deterministic norm  */
    int surface_prolong;    /* 1: also correct the last row (see qo_prolongate) */
    int coarse_solve;       /* 1: exact solve on the coarsest level (qo_coarse_solve) */
} qo_mg;

int  qo_mg_init(qo_mg *m, int ni, int nk, double dh, const double *mu_equi,
                int n_levels, int nu_pre, int nu_post, int nu_coarse);
void qo_mg_free(qo_mg *m);
/* Depth metric J = dz/dzeta per staggered row of mu_equi (2(nk+2)-1 values;
 * NULL: uniform). */
void qo_mg_set_metric(qo_mg *m, int nk, const double *jrow);

/* single kernels, restated (odeSolver.cpp:757-1043) */
void qo_rbgs(const qo_mg *m, double *u, const double *f, int level, int phase);
void qo_residual(const qo_mg *m, double *r, const double *u, const double *f, int level);
void qo_restriction(const qo_mg *m, double *r2, const double *r, double *e2, int level);
void qo_prolongate(const qo_mg *m, double *u, const double *e2, int level);
void qo_smooth(const qo_mg *m, double *u, const double *f, int level, int nsweeps);
void qo_vcycle(qo_mg *m, double *u, const double *f, int level);
double qo_norm2(qo_mg *m, const double *r, int level);

/* residual norm of the zero-interior guess (columns 0 and K-1 of u kept) */
double qo_r0_norm(qo_mg *m, const double *u, int level);

/* multigrid(): iterate V-cycles until ||r|| <= tol (tol_mode 0: absolute as
 * odeSolver.cpp:689-705; 1: relative to qo_r0_norm).  max_cycles <= 0 means
 * no cap, as in the reference.  Returns cycles done; *rnorm = final norm. */
int qo_multigrid(qo_mg *m, double *u, const double *f, int tol_mode, double tol,
                 int max_cycles, double *rnorm, double *r0norm);

/* --------------- boundary / ghosts (odeSolver.cpp:612-650,1150-1188) ---- */
void qo_extend_crew(int ni, int nk, double *U);
void qo_set_boundary(int ni, int nk, double *U, const double *slip,
                     const double *slip_shift, double vini, double t_elapsed,
                     double ratio, double dt);
void qo_pack(int ni, int nk, const double *U, double *u);   /* :669-677 */
void qo_unpack(int ni, int nk, const double *u, double *U); /* :708-716 */

/* --------------- fault physics (fault.cpp:139-232, odeSolver.cpp:1190) -- */
void qo_eval_stress_on_fault(int ni, int nk, double dh, const double *U,
                             const double *mu_node, const double *Tau_n0,
                             double *Ts, double *Tn);
/* NRsearch with the project's tau0 prestress (fb = Ts + tau0; tau0 == NULL
 * reproduces the reference exactly).  V holds the seed on entry (the
 * reference's rk4.V_f) and the slip rate on exit.  Returns 0, or -1-k for a
 * node whose friction stayed NaN (the reference exit(0)s there). iters, if
 * non-NULL, receives the Newton iteration count per node. */
int qo_nrsearch(int nk, const double *Ts, const double *Tn, const double *tau0,
                const double *a, const double *eta, const double *psi,
                double V0, double *V, int *iters);
void qo_cal_dpsi(int nk, const double *psi, const double *b, const double *V,
                 double f0, double V0, double L, double *dpsi);
double qo_compute_error(int nk, const double *slip3, const double *psi3,
                        const double *slip4, const double *psi4);
double qo_compute_step_size(int it, double dt, double mindt, double maxdt,
                            double totErr, double totTol, const double errA[2]);

/* --------------- SetMedium homogenisation (odeSolver.cpp:134-601) ------- */
/* Builds mu_half / mu_equi ((2nx-1)*(2nz-1)) from the ghosted node array
 * mu_node (interior nodes set).  The reference leaves mu_matrix[1][1]
 * unset at odeSolver.cpp:434-436; this restatement sets it to the node it
 * evidently means (mu_half[index3 + 2]). */
void qo_set_medium(int ni, int nk, const double *mu_node, double *mu_half,
                   double *mu_equi);
/* interp_2d (x-edge stencil, 3x4) and interp2_2d (z-edge stencil, 4x3) */
double qo_interp_xedge(const double *z12, double xi, double yi);
double qo_interp_zedge(const double *z12, double xi, double yi);

/* --------------- RK43 driver (odeSolver.cpp:1277-1674) ----------------- */
typedef struct qo_sim qo_sim;   /* opaque */

/* tol_mode / tol / max_cycles as qo_multigrid. */
qo_sim *qo_sim_create(int ni, int nk, double dh, const double *mu_node,
                      const double *mu_equi, int n_levels, int nu_pre,
                      int nu_post, int nu_coarse, int tol_mode, double tol,
                      int max_cycles);
void qo_sim_free(qo_sim *s);
/* Fault arrays are nz long (reference layout); tau0 may be NULL. */
void qo_sim_set_fault(qo_sim *s, const double *a, const double *b,
                      const double *eta, const double *Tau_n0,
                      const double *SlipShift, const double *tau0,
                      const double *Slip, const double *psi, double f0,
                      double V0, double L, double Vini);
void qo_sim_set_params(qo_sim *s, double tmax, double ini_dt, double mindt,
                       double maxdt, double totTol, int maxNumSteps);
void qo_sim_set_U(qo_sim *s, const double *U);       /* ghosted nx*nz */
void qo_sim_set_surface_prolong(qo_sim *s, int v);
void qo_sim_set_metric(qo_sim *s, const double *jrow);
void qo_sim_set_coarse_solve(qo_sim *s, int v);
/* The pre-loop part of RK43 (odeSolver.cpp:1363, 1428-1439). */
int  qo_sim_start(qo_sim *s);
/* The elliptic solve of ode_solve() by another implementation: called with
 * the packed compact u (nk rows x ni columns, host memory; columns 0 and
 * ni-1 the Dirichlet data) in place of qo_multigrid, it solves u in place
 * and returns the V-cycles it took (and the final norm in *rnorm).  Used to
 * run the reference's own GPU multigrid kernels under this RK43 loop, as
 * the reference's ode_solve() does (odeSolver.cpp:605-720). */
typedef int (*qo_solve_hook)(void *ctx, double *u, int ni, int nk, double *rnorm);
void qo_sim_set_solve_hook(qo_sim *s, qo_solve_hook fn, void *ctx);
/* Restart from the fault state alone (Slip, psi and the loop's scalars):
 * the refresh solve and fault update that end an accepted step
 * (odeSolver.cpp:1605-1619), from the current U as the guess. */
int  qo_sim_resume(qo_sim *s, const double *Slip, const double *psi, double t,
                   double dt, double errA0, double errA1, int it);
/* One pass of the outer while-loop body (odeSolver.cpp:1462-1636). */
int  qo_sim_step(qo_sim *s);
/* Full state read-back.  Any pointer may be NULL.  V is f1.V_f. */
void qo_sim_get(const qo_sim *s, double *U, double *Slip, double *psi,
                double *V, double *Ts, double *dpsi);
/* scalars: t, dt, errA0, errA1; counters: it, solves, vcycles, attempts,
 * newton_iters, status */
void qo_sim_scalars(const qo_sim *s, double *dvals4, long long *ivals6);
/* Restore the time-stepping scalars (checkpoint resume). */
void qo_sim_set_scalars(qo_sim *s, double t, double dt, double errA0,
                        double errA1, int it);

int qo_num_threads(void);
void qo_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
