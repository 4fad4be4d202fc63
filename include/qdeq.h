/*
 * qdeq.h -- C ABI of the GB300 (sm_103a) quasi-dynamic earthquake-cycle hot
 * path: the per-stage pipeline of QDEqCycle_FDM's adaptive RK43 loop
 * (multigrid u-solve, fault shear stress, Newton solve for slip rate, aging
 * law, RK stage combination / error estimate / step control).
 *
 * The reference has no plugin or FFI layer; its interface is the set of C++
 * free functions in functions.h:11-45, taking struct.h structs by value with
 * borrowed Real* arrays.  Each entry point below names the reference function
 * it replaces.  Conventions:
 *   - plain pointers and sizes only; every array pointer is HOST memory
 *     unless the name says "device";
 *   - arrays use the reference's layouts: ghosted fields (U, mu_node) are
 *     nx*nz doubles indexed i + k*nx with nx = ni+2, nz = nk+2 (struct.h,
 *     odeSolver.cpp:24-38); fault vectors are nz doubles whose entries
 *     1..nk are used (Alloc.cpp:3-42); mu_equi is (2nx-1)*(2nz-1) doubles
 *     (odeSolver.cpp:47,337-589);
 *   - every call returns a status (QD_OK = 0); qd_last_error() describes the
 *     last failure of the calling thread.  Nothing calls exit().
 *   - a solver owns one CUDA stream and all of its device memory; calls on
 *     one solver are serialised by the caller.  The reference runs one host
 *     thread on the default stream.
 */
#ifndef QDEQ_H
#define QDEQ_H

#ifdef __cplusplus
extern "C" {
#endif

#define QDEQ_ABI_VERSION 1

/* status codes */
#define QD_OK 0
#define QD_ERR_ARG 1            /* bad argument or size                      */
#define QD_ERR_CUDA 2           /* CUDA runtime error                        */
#define QD_ERR_NOMEM 3          /* device allocation failed                  */
#define QD_ERR_NOT_CONVERGED 4  /* multigrid hit max_cycles above tolerance  */
#define QD_ERR_NEWTON 5         /* Newton for V gave NaN/no root (the
                                   reference exit(0)s: fault.cpp:211-225)    */
#define QD_ERR_STATE 6          /* call out of order (e.g. no fault set up)  */

/* tolerance modes */
#define QD_TOL_ABS 0            /* ||r||2 <= tol, as odeSolver.cpp:689-705   */
#define QD_TOL_REL 1            /* ||r||2 <= tol * ||r(u_interior = 0)||2    */

/* precision of the multigrid cycles */
#define QD_PREC_FP64 0          /* FP64 V-cycles (the drop-in)               */
#define QD_PREC_MIXED 1         /* FP32 V-cycles inside FP64 iterative
                                   refinement: FP64 u and update, residual
                                   in double-float (48-bit) arithmetic       */

/* Ceiling on the V-cycles of one solve run as a CUDA graph when max_cycles
 * is <= 0: the graph's loop is decided on the device, where no host check
 * could stop a solve whose tolerance is out of reach (an absolute tolerance
 * below the round-off floor of a large grid, or a refinement that stalls). */
#define QD_SOLVE_GRAPH_MAX_CYCLES 10000

typedef struct qd_solver qd_solver;

/* Multigrid schedule.  The reference hard-codes n_levels = 6, V(32,32) with
 * 32 sweeps on the coarsest level, plain red-black Gauss-Seidel and an
 * absolute 1e-9 residual norm (odeSolver.cpp:2-4,689). */
typedef struct qd_mg_options {
    int n_levels;
    int nu_pre;       /* red+black sweeps before the coarse correction       */
    int nu_post;      /* ... and after it                                    */
    int nu_coarse;    /* sweeps on the coarsest level                        */
    int tol_mode;     /* QD_TOL_ABS or QD_TOL_REL                            */
    double tol;
    int max_cycles;   /* V-cycles per solve before QD_ERR_NOT_CONVERGED
                         (<= 0: no cap in the host-driven loop, as the
                         reference; a solve run as a CUDA graph, the
                         default, loops on the device and stops after
                         QD_SOLVE_GRAPH_MAX_CYCLES instead)                 */
    int precision;    /* QD_PREC_FP64 or QD_PREC_MIXED                       */
    int surface_prolong; /* 0: as prolongate_kernel (odeSolver.cpp:1034), the
                         last row (the free surface) gets no coarse-grid
                         correction; 1: it gets the coincident coarse row's
                         correction too (same discrete solution, about 5x
                         fewer V(2,2) cycles)                                */
    int coarse_solve;    /* 0: nu_coarse red+black sweeps on the coarsest level,
                         as vcycle() (odeSolver.cpp:1103-1107); 1: exact
                         solve there with a dense inverse built at set-up
                         (coarsest level of at most 1024 unknowns)           */
} qd_mg_options;

/* Time-stepping parameters (PARAMS, struct.h:12-38; SetParams.cpp:14-21). */
typedef struct qd_rk43_params {
    double tmax;      /* s */
    double ini_dt;
    double mindt;
    double maxdt;
    double totTol;
    int maxNumSteps;
} qd_rk43_params;

/* Counters of one solver since creation. */
typedef struct qd_stats {
    long long solves;        /* elliptic solves (ode_solve calls)            */
    long long vcycles;       /* V-cycles (FP32 ones in mixed precision)      */
    long long attempts;      /* RK43 attempts (accepted + rejected)          */
    long long steps;         /* accepted RK43 steps                          */
    long long newton_iters;  /* Newton iterations, summed over nodes         */
    long long kernel_launches; /* kernels this library launched              */
    long long net_solves;    /* solves whose guess the attached network
                                corrected (prediction mode: only solves
                                whose guess missed the tolerance)          */
    double net_cycles_needed; /* over those solves: the V-cycles their
                                guesses would have needed (from the
                                measured reduction per cycle) ...          */
    double net_cycles_taken;  /* ... and the V-cycles they took            */
    long long smooth_corrections; /* level-0 smoothing passes that replaced
                                a V-cycle (qd_set_smooth_correction)       */
    long long net_armed_solves; /* solves that carried the attached
                                network's conditional correction (not on
                                standby), whether or not it ran            */
} qd_stats;

const char *qd_version(void);
const char *qd_last_error(void);
/* The reference's schedule: 6 levels, V(32,32), 32 coarse sweeps, absolute
 * 1e-9, no cap, FP64. */
void qd_default_options(qd_mg_options *opt);

/* ---------------------------------------------------------------------
 * Set-up.  Replaces RK43's GPU initialisation (odeSolver.cpp:1365-1425):
 * level tables, cudaMalloc of the level buffers, H2D of mu_equi.
 * mu_equi: (2nx-1)*(2nz-1) face moduli (GPa); mu_node: nx*nz node moduli
 * (only the fault column i = 1 is used, by the stress extraction,
 * fault.cpp:153).  (ni-1) and (nk-1) must be divisible by 2^(n_levels-1).
 * ------------------------------------------------------------------- */
int qd_solver_create(int ni, int nk, double dh, const double *mu_equi,
                     const double *mu_node, const qd_mg_options *opt,
                     qd_solver **out);
/* The same on a grid stretched in depth (no counterpart in the reference,
 * whose grid is uniform, coord.cpp:18,27): z = z(zeta) with the
 * computational coordinate zeta uniform, spacing dh like x, and the
 * operator div(mu grad u) in its conservative mapped form
 *   J d/dx(mu du/dx) + d/dzeta((mu / J) du/dzeta),   J = dz/dzeta,
 * i.e. x-face moduli mu J and z-face moduli mu / J on the uniform
 * computational grid.  jrow: J at every staggered row of mu_equi (2nz-1
 * values: even rows at nodes, odd rows at faces, the ghost rows mirrored),
 * all positive; NULL gives qd_solver_create.  The fault stress (a derivative
 * in x) and everything else are unchanged. */
int qd_solver_create_mapped(int ni, int nk, double dh, const double *mu_equi,
                            const double *mu_node, const double *jrow,
                            const qd_mg_options *opt, qd_solver **out);
int qd_solver_destroy(qd_solver *s);
int qd_solver_set_options(qd_solver *s, const qd_mg_options *opt);
int qd_get_stats(qd_solver *s, qd_stats *st);
/* The solver's CUDA stream (a cudaStream_t), for callers that order their
 * own work or CUDA events after the solver's. */
void *qd_solver_stream(qd_solver *s);

/* SetMedium's homogenisation (odeSolver.cpp:337-589) on the GPU: the harmonic
 * mean of 400 Lagrange-interpolated samples per cell face.  mu_node is the
 * ghosted nx*nz node modulus with the interior set; writes mu_equi.  Needs
 * no solver. */
int qd_set_medium(int ni, int nk, const double *mu_node, double *mu_equi);

/* ---------------------------------------------------------------------
 * Displacement field.  The device keeps u compact (nk rows x ni columns)
 * for the whole run; these copy it to and from the reference's ghosted
 * host array (replacing the pack/unpack of odeSolver.cpp:669-677,707-716
 * and extend_crew, :612-650).
 * ------------------------------------------------------------------- */
int qd_upload_u(qd_solver *s, const double *U);
int qd_download_u(qd_solver *s, double *U);

/* One elliptic solve on the device-resident u: multigrid() + extend_crew()
 * (ode_solve, odeSolver.cpp:605-720).  Columns 0 and ni-1 of u are the
 * Dirichlet data.  cycles / rnorm / r0norm may be NULL. */
int qd_ode_solve(qd_solver *s, int *cycles, double *rnorm, double *r0norm);

/* ode_solve with the reference's host round trip: U (ghosted, host) in,
 * solved U with ghosts out. */
int qd_ode_solve_host(qd_solver *s, double *U, int *cycles, double *rnorm);

/* Individual multigrid steps on the level-0 field, for parity tests:
 * nsweeps red+black sweeps (smooth(), odeSolver.cpp:741-755); one V-cycle
 * (vcycle(), :1101-1147); the level-0 residual norm (calcuDelta_dev +
 * cublasDnrm2, :693-694). */
int qd_mg_smooth(qd_solver *s, int nsweeps);
int qd_mg_vcycle(qd_solver *s);
int qd_mg_residual_norm(qd_solver *s, double *rnorm);

/* Per-launch device time of one kernel of the V-cycle that the solver's
 * precision runs (inside a solve they run in a CUDA graph, out of reach of
 * per-kernel events): the kernel is launched `reps` times back to back on
 * the solver's stream between two CUDA events and *us receives the mean
 * microseconds per launch.  The launches change the solver's state (they
 * smooth, restrict and add corrections), so use it after a run, for
 * roofline measurements.  No counterpart in the reference. */
#define QD_KERNEL_DOWN0    0   /* level-0 pre-smoothing + residual + restriction tile kernel */
#define QD_KERNEL_UP0      1   /* level-0 prolongation + post-smoothing tile kernel (final pass) */
#define QD_KERNEL_RESIDUAL 2   /* FP64 level-0 residual -> FP32 right-hand side + norm (mixed) */
#define QD_KERNEL_TAIL     3   /* single-CTA coarse tail */
int qd_mg_time_kernel(qd_solver *s, int kernel, int reps, double *us);

/* Test hook for the bounded waits of the shared-memory staging pipelines
 * (every mbarrier wait of the multigrid tile kernels and the U-Net's
 * convolutions gives up after a fixed number of polls instead of spinning
 * forever): one kernel on the solver's stream waits on an mbarrier that
 * nothing completes, gives up after `polls` polls (1 .. 4,194,304, the
 * pipelines' own limit), records the timeout in the solver's status word and
 * returns.  The call then reports it as a solver call does after a staging
 * wait gave up: QD_ERR_CUDA, with qd_last_error() naming the staging.  The
 * CUDA context stays usable; the status word stays set until the next
 * qd_rk43_start.  No counterpart in the reference. */
int qd_probe_bounded_wait(qd_solver *s, int polls);

/* The binary64 -> binary32 rounding (to nearest, ties to even) that the
 * learned warm start's input kernels perform on the device's integer pipes,
 * applied to n host values (a device round trip), so that tests can hold it
 * to IEEE conversion on the host.  No counterpart in the reference. */
int qd_convert_f64_to_f32(const double *in, float *out, int n);

/* The binary64 -> double-float split (x = hi + lo, two binary32 values,
 * to within 2^-47 |x|) that the mixed-precision residual kernel performs on
 * the device's integer pipes, applied to n host values (a device round
 * trip), for tests.  No counterpart in the reference. */
int qd_split_f64(const double *in, float *hi, float *lo, int n);

/* The level-0 residual norm ||0 - A u||2 that qd_mg_residual_norm returns,
 * for a caller that cannot allocate device memory: a host framework that
 * owns every device byte (its own allocator, or a budget fixed at start-up),
 * or code where a cudaMalloc would synchronise the device in the middle of
 * its own work.  It needs no solver and allocates nothing: u (nk rows x ni
 * columns), cx and cz (the face moduli of a solver's level 0 -- cx[j][k]
 * between columns k and k+1, cz[j][k] for j = 0..nk between rows j-1 and j)
 * are DEVICE arrays the caller owns, with a row pitch of `pitch` doubles;
 * dh is the grid spacing; the work runs on `stream` (a cudaStream_t; NULL
 * for the default stream) and *rnorm (host) receives the norm.
 * The block partial sums live in a file-scope device array of 66,178
 * doubles (517 KB) that every GPU using this library keeps until the
 * process exits; grids of more than 4097 rows or 4097 columns are rejected with
 * QD_ERR_ARG.  The first call on each device looks up that array's device
 * address and keeps it.  All calls share the array: calls that overlap on the GPU (two streams, two host threads)
 * race and must be serialised by the caller.  This entry point has no
 * counterpart in the reference. */
int qd_residual_norm_noalloc(const double *u, const double *cx, const double *cz, int nk, int ni,
                             int pitch, double dh, void *stream, double *rnorm);

/* ---------------------------------------------------------------------
 * Fault.  Arrays are nz long (entries 1..nk used).  tau0 (MPa) is added to
 * the stress the Newton solve balances; pass NULL for the reference's
 * behaviour (no prestress).  Scalars are RATE_STATE_LAW's f0, V0, L, Vini
 * (Alloc.cpp:27-31).
 * ------------------------------------------------------------------- */
int qd_fault_setup(qd_solver *s, const double *a, const double *b,
                   const double *eta, const double *Tau_n0,
                   const double *SlipShift, const double *tau0, double f0,
                   double V0, double L, double Vini);

/* setBoundary (odeSolver.cpp:1150-1188) on the device u: fault column
 * u = slip/2, remote column u = Vini (t + ratio dt)/2 + SlipShift. */
int qd_set_boundary(qd_solver *s, const double *slip, double t_elapsed,
                    double ratio, double dt);

/* eval_stress_on_fault (fault.cpp:139-164) from the device u: Ts (MPa) and
 * Tn = Tau_n0.  Either output may be NULL. */
int qd_eval_stress_on_fault(qd_solver *s, double *Ts, double *Tn);

/* NRsearch (fault.cpp:169-232): slip rate from Ts (+tau0), psi and the
 * seed in V (overwritten with the result).  One thread per fault node,
 * Newton in x = asinh(V e^{psi/a} / 2V0) safeguarded by a sign bracket;
 * from the reference's seed the iterates are the reference's.  iters may
 * be NULL (else nz ints). */
int qd_nrsearch(qd_solver *s, const double *Ts, const double *psi, double *V,
                int *iters);

/* cal_dpsi (odeSolver.cpp:1190-1206): aging law. */
int qd_cal_dpsi(qd_solver *s, const double *psi, const double *V, double *dpsi);

/* ---------------------------------------------------------------------
 * RK43 (odeSolver.cpp:1277-1674) with the whole state on the device.
 * qd_rk43_start runs the pre-loop part (initial solve, stress, Newton,
 * aging law: :1363,1428-1439) from Slip/psi and the uploaded u;
 * qd_rk43_step runs nsteps passes of the outer while-loop body
 * (:1462-1636), stopping early at tmax or maxNumSteps.
 * ------------------------------------------------------------------- */
int qd_rk43_start(qd_solver *s, const qd_rk43_params *p, const double *Slip,
                  const double *psi);
int qd_rk43_step(qd_solver *s, int nsteps, int *steps_done);
/* qd_rk43_step on a state that lives on the host, the way the reference's
 * RK43 holds it: Slip, psi, V (= f1.V_f), dpsi (= f1.dpsi) (nz arrays) and
 * the ghosted nz x nx field U are uploaded, nsteps steps are taken, and all
 * five, with Ts (nz, may be NULL), are written back; state4 holds
 * {t, dt, errA0, errA1} and *it the accepted step count, read and updated.
 * The same as qd_rk43_set_state, qd_upload_u, qd_rk43_step,
 * qd_rk43_get_state and qd_download_u in turn, with the transfers queued
 * behind one another and one host wait instead of five (pinned host
 * buffers let the copies run asynchronously).  No counterpart in the
 * reference. */
int qd_rk43_step_host(qd_solver *s, int nsteps, double *Slip, double *psi, double *V,
                      double *dpsi, double *Ts, double *U, double *state4, int *it,
                      int *steps_done);
/* Restart from the fault state alone (a compact checkpoint: Slip and psi,
 * nz arrays, and the loop's scalars t, dt, errA0, errA1 and the accepted
 * step count it): the state an accepted step leaves behind is Slip, psi,
 * t, dt and the error history, and everything else follows from them.  Sets
 * the boundary data from Slip at t, solves from the device u as it stands
 * (upload a guess first, e.g. the last known u or zero), then takes the
 * stress, Newton (from the zero seed) and aging law -- the refresh solve of
 * a commit (odeSolver.cpp:1605-1619) -- and keeps dt; the next qd_rk43_step
 * continues from there.  The solution history is cleared.  No counterpart
 * in the reference, which always starts from t = 0. */
int qd_rk43_resume(qd_solver *s, const qd_rk43_params *p, const double *Slip,
                   const double *psi, double t, double dt, double errA0,
                   double errA1, int it);
/* Batched ensemble: advance n independent, started solvers (any grids and
 * parameters, each with its own adaptive dt) by nsteps accepted steps each,
 * interleaving their GPU work: every instance's attempt (stages 2-6 and the
 * error estimate) is queued on its own stream before the host waits on any,
 * so the kernels of small instances fill the GPU together.  Each instance
 * follows exactly the operations qd_rk43_step would run on it.  An instance
 * at tmax or maxNumSteps stops; steps_done (n entries, may be NULL) gets the
 * steps each took.  No counterpart in the reference, which runs one
 * simulation per process. */
int qd_ensemble_step(qd_solver **s, int n, int nsteps, int *steps_done);
/* State read-back (any pointer may be NULL): Slip, psi, V (= f1.V_f),
 * Ts, dpsi (= f1.dpsi). */
int qd_rk43_get_state(qd_solver *s, double *Slip, double *psi, double *V,
                      double *Ts, double *dpsi);
/* Scalars: d[0] = t, d[1] = dt, d[2..3] = errA; it = accepted steps. */
int qd_rk43_get_scalars(qd_solver *s, double *d4, int *it);
/* Overwrite the state (checkpoint resume / host-driven stepping): Slip, psi,
 * V, dpsi are nz arrays (V/dpsi: f1 after the last accepted step). */
int qd_rk43_set_state(qd_solver *s, const double *Slip, const double *psi,
                      const double *V, const double *dpsi, double t, double dt,
                      double errA0, double errA1, int it);

/* Autotuner.  Times every candidate smoother schedule (nu_pre, nu_post in
 * {1,1 2,2 3,3 4,4 1,2 2,1 2,3 3,2}) and pair of tile box widths of the
 * descending and ascending tile kernels ({64, 96, 128} columns each) on
 * `reps` solves to the solver's tolerance, keeps the fastest (options and
 * tiles), and restores u and the solve counters.  The timed solves are the
 * run's own kind: with a solution history holding at least three solutions,
 * its last stored solve replayed from the guess of the solutions before it
 * (when that solve takes a V-cycle); otherwise the current boundary data
 * from a zero interior.  The reference's schedule is fixed (odeSolver.cpp:2-4).
 * n_levels, precision and the tolerance are not changed.  out may be NULL. */
typedef struct qd_tuning {
    int nu_pre, nu_post;       /* the schedule picked                         */
    int box_up, box_down;      /* the tile box widths picked (columns)        */
    double us_best;            /* its mean time per solve                     */
    double us_initial;         /* the same for the settings before tuning     */
    int cycles_best, cycles_initial;   /* V-cycles of those solves            */
    int candidates;            /* settings that converged and were timed      */
    int replayed;              /* 1: timed on the replayed history solve,
                                  0: on solves from a zero interior          */
} qd_tuning;
int qd_autotune(qd_solver *s, int reps, qd_tuning *out);
/* Staged box widths of the tile kernels (multiples of 16 in 32..256; 0: the
 * default 64).  qd_autotune sets them; this sets them directly. */
int qd_set_tiles(qd_solver *s, int box_up, int box_down);

/* Initial guess of the RK43 driver's stage solves from the solution history
 * (no counterpart in the reference, which starts every solve from the last
 * solution, odeSolver.cpp:669-677).  With m >= 2 the solver keeps its last m
 * level-0 solutions (m x 8*nk*pitch bytes of device memory) and starts each
 * stage solve from A + sum_k c_k (S_k - A): A the latest solution, S_k the
 * earlier ones, c the least-squares fit of the stage's new fault and far
 * boundary columns by theirs.  The multigrid still iterates to the same
 * residual tolerance; only the V-cycle count changes.  m = 0 or 1: off (the
 * default).  m at most 8.  The stored solutions are solutions of the
 * solver's fixed operator, so they stay valid when u or the RK state is
 * replaced (qd_upload_u, qd_rk43_set_state); a new run (qd_rk43_start) and
 * qd_checkpoint_load clear them, and a checkpoint file does not hold them. */
int qd_set_solution_history(qd_solver *s, int m);
/* Start of the Newton solve for slip rate where the seed is the
 * reference's zero (every RK stage, fault.cpp:180-228 with
 * odeSolver.cpp:1484-1488).  mode 0 (the default): x = 0, the reference's
 * iterates.  mode 1: x from a binary32 Newton solve of the log form of the
 * same equation, then the same FP64 iteration and stopping rule, which end
 * at the same root (to the rule's 1e-10) in two or three FP64 steps where
 * the reference's start takes up to eleven near a rupture front.  The
 * iteration count the solver reports is then that of the FP64 steps.  No
 * counterpart in the reference. */
int qd_set_newton_start(qd_solver *s, int mode);
/* Red-black sweeps before and after the coarse-grid correction on the
 * levels the single-CTA coarse tail runs (those of at most 65 rows): n >= 1
 * sets both to n; 0 (the default) keeps the fine levels' nu_pre and
 * nu_post, the reference's schedule.  On those levels a V-cycle is bound by
 * one SM's barriers, and with the exact coarsest solve fewer sweeps there
 * leave the cycle's reduction nearly unchanged.  No counterpart in the
 * reference. */
int qd_set_tail_sweeps(qd_solver *s, int n);
/* Mixed precision only: after a V-cycle that leaves ||r|| above the
 * threshold by at most `ratio`, the next correction of the solve is a
 * level-0 smoothing pass (four red-black sweeps on the correction equation
 * from zero, one kernel) instead of a V-cycle; at most one such pass in a
 * row, and the solve still stops only at the same tolerance.  A V-cycle
 * leaves a residual whose norm is mostly rough components, which the pass
 * removes: at 1025^2 it cuts ||r|| to about a third, so ratios up to about
 * 2.5 finish the solve with it.  ratio 0 (the default): off.  Counted in
 * qd_stats.smooth_corrections, not in vcycles.  No counterpart in the
 * reference. */
int qd_set_smooth_correction(qd_solver *s, double ratio);
/* The last fit: coef[0..6] the coefficients of the earlier solutions
 * (newest first), coef[7] the fit's boundary misfit over the change from
 * the latest solution's boundary data (1: no gain); *nd coefficients are
 * in use.  Synchronises the solver's stream. */
int qd_solution_history_fit(qd_solver *s, double *coef, int *nd);

/* ---------------------------------------------------------------------
 * Files.
 * ------------------------------------------------------------------- */
/* The initial displacement file RK43 reads (odeSolver.cpp:96-128): ni * nk
 * doubles, column index fastest, the interior nodes of the ghosted
 * (ni+2) x (nk+2) array U.  load fills U's interior (ghosts untouched) and
 * fails with QD_ERR_ARG on a short file, where the reference prints
 * "Read error!" and continues; save writes that layout from U's interior. */
int qd_load_initial_u(const char *path, int ni, int nk, double *U);
int qd_save_initial_u(const char *path, int ni, int nk, const double *U);

/* Snapshot record of the current state in the reference's format:
 * full = 1 is the first record (odeSolver.cpp:1442-1456: t, V, Slip, Ts, psi,
 * U with ghosts, Tn, a, b, dt), full = 0 the periodic one (:1638-1652: t, V,
 * Slip, Ts, psi, dt).  With async = 1 the device-to-host copies are queued on
 * the solver's stream and a host thread writes the file once they land, so
 * the solver keeps stepping; one snapshot is in flight per solver (a new one
 * first waits for the last).  qd_snapshot_wait joins it and returns its
 * status.  No counterpart in the reference beyond the record layout. */
int qd_snapshot(qd_solver *s, const char *path, int full, int async);
int qd_snapshot_wait(qd_solver *s);

/* Checkpoint / restart: every piece of state the next accepted step reads
 * (Slip, psi, V, Ts, dpsi, t, dt, the error history, the step count, the
 * time-stepping parameters and u), so that a run loaded from a checkpoint
 * continues bit for bit as the saved run would have; loading replaces
 * qd_rk43_start.  The solver loading it must have the same grid, medium,
 * fault set-up and multigrid options.  File: "QDEQCKP1", int32 ni, nk, it,
 * maxNumSteps, doubles t, dt, errA0, errA1, tmax, ini_dt, mindt, maxdt,
 * totTol, then Slip, psi, V, Ts, dpsi (nz each) and u (nk rows of ni).  No
 * counterpart in the reference. */
int qd_checkpoint_save(qd_solver *s, const char *path);
int qd_checkpoint_load(qd_solver *s, const char *path);

#ifdef __cplusplus
}
#endif
#endif /* QDEQ_H */
