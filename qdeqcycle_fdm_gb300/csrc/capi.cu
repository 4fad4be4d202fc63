// capi.cu -- the extern "C" boundary (include/qdeq.h) and the RK43 host
// driver.  The driver keeps the reference's control flow
// (odeSolver.cpp:1277-1674) on the host -- attempt loop, step-size control,
// commit -- and runs every per-node and per-grid-point operation on the
// device; the only device-to-host traffic per attempt is the error estimate,
// and per V-cycle the residual norm.
#include <math.h>

#include <cmath>
#include <stdarg.h>
#include <string.h>

#include <vector>

#include "qdeq_internal.cuh"
#include "tma.cuh"

namespace qd {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

static int check_opts(const qd_mg_options *o) {
    if (!o || o->n_levels < 1 || o->n_levels > QD_MAXLEV || o->nu_pre < 0 || o->nu_post < 0 ||
        o->nu_coarse < 0 || (o->tol_mode != QD_TOL_ABS && o->tol_mode != QD_TOL_REL) ||
        !(o->tol > 0.0) || (o->precision != QD_PREC_FP64 && o->precision != QD_PREC_MIXED) ||
        (o->surface_prolong != 0 && o->surface_prolong != 1) ||
        (o->coarse_solve != 0 && o->coarse_solve != 1)) {
        set_error("invalid multigrid options");
        return QD_ERR_ARG;
    }
    return QD_OK;
}

// The step-size controller (computeStepSize, odeSolver.cpp:1241-1271).  A
// zero in the error history (an accepted step whose two embedded solutions
// agreed to the last bit) makes the reference's PID branch return mindt or
// NaN; with a zero there the elementary controller the reference uses for
// its first steps (:1254-1257) is taken instead.
static double step_size(int it, double dt, const qd_rk43_params &P, double totErr,
                        const double errA[2]) {
    const double ord = 4.0, kappa = 0.9;
    const double alpha = 0.49 / ord, beta = 0.34 / ord, gamma = 0.1 / ord;
    const double totTol = P.totTol;
    double stepRatio;
    if (it < 4 || errA[0] == 0.0 || errA[1] == 0.0)
        stepRatio = kappa * pow(totTol / totErr, 1.0 / (1.0 + ord));
    else
        stepRatio = kappa * pow(totTol / totErr, alpha) * pow(errA[0] / totTol, beta) *
                    pow(totTol / errA[1], gamma);
    double deltaT = stepRatio * dt;
    deltaT = (dt * 5.0 <= deltaT) ? dt * 5.0 : deltaT;
    deltaT = (P.maxdt <= deltaT) ? P.maxdt : deltaT;
    deltaT = (P.mindt >= deltaT) ? P.mindt : deltaT;
    return deltaT;
}

// Multigrid failures the device recorded since the flag was last cleared
static int solve_flag_error(const SolveState &st) {
    if (st.flag & 1) {
        set_error("multigrid: residual norm is not finite (%d cycles)", st.cycles);
        return QD_ERR_NOT_CONVERGED;
    }
    if (st.flag & 2) {
        set_error("multigrid: cycle cap reached, ||r|| = %.3e > %.3e", st.delta, st.thr);
        return QD_ERR_NOT_CONVERGED;
    }
    return QD_OK;
}

// Failures the device kernels recorded in the status word: a bounded wait
// that gave up, or a Newton solve with no finite root (where the reference
// exit(0)s, fault.cpp:211-225)
static int status_flag_error(const DevStatus &d) {
    if (d.flags & ST_TMA_TIMEOUT) {
        set_error("a multigrid kernel's shared-memory staging did not complete (flags %u)", d.flags);
        return QD_ERR_CUDA;
    }
    if (d.flags & (ST_NEWTON_NAN | ST_NEWTON_CAP)) {
        set_error("Newton for slip rate failed at fault node %d (flags %u)", d.bad_node, d.flags);
        return QD_ERR_NEWTON;
    }
    return QD_OK;
}

static int check_status(qd_solver *s) {
    QD_CUDA(cudaMemcpyAsync(s->h_status, s->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost,
                            s->stream));
    SolveState st;
    QD_TRY(solve_state_read(s, &st));   // synchronises the stream
    QD_TRY(solve_flag_error(st));
    return status_flag_error(*s->h_status);
}

static int reset_status(qd_solver *s) {
    DevStatus z;
    z.flags = 0;
    z.bad_node = -1;
    *s->h_status = z;
    QD_CUDA(cudaMemcpyAsync(s->d_status, s->h_status, sizeof(DevStatus), cudaMemcpyHostToDevice,
                            s->stream));
    return QD_OK;
}

// one stage: boundary data, elliptic solve, stress/Newton/aging law, all
// enqueued on the solver's stream without waiting
static int stage(qd_solver *s, int st, double ratio, bool commit = false) {
    QD_TRY(warm_start_before_boundary(s));     // no-ops without an attached network
    QD_TRY(launch_stage_boundary(s, st, ratio, true, commit));   // + the history fit when enabled
    QD_TRY(history_apply(s, warm_start_bc_buffer(s)));   // no-op unless enabled
    QD_TRY(warm_start_after_boundary(s));
    QD_TRY(mg_solve_async(s));
    QD_TRY(warm_start_after_solve(s));
    CopyJob push;
    QD_TRY(history_push_job(s, &push));   // stored by the fault stage's extra blocks
    return launch_fault(s, st, push);
}

static int rk_start(qd_solver *s) {
    s->dt = s->P.ini_dt;                                          // :1363
    QD_TRY(reset_status(s));
    QD_TRY(solve_state_clear_flag(s));
    QD_TRY(stage(s, 1, 0.0));                                     // :1428-1437
    QD_TRY(check_status(s));
    s->started = 1;
    return QD_OK;
}

// The outer while-loop body, odeSolver.cpp:1464-1636, in phases that only
// enqueue work (step_begin, attempt_enqueue, commit_enqueue) and phases that
// wait for it (attempt_finish, commit_finish), so that several solvers can
// interleave their GPU work (qd_ensemble_step).
struct RkTableau {
    double c[7], b[7], hb[7], a[7][7];
};
static const double *rk_c() {
    // built once, thread-safely (function-local static), for every solver
    static const RkTableau t = [] {
        RkTableau x;
        rk_tableau(x.c, x.b, x.hb, x.a);
        return x;
    }();
    return t.c;
}

// The solve's failure flags are not cleared between steps: every flag is a
// failure the step reports, after which the run restarts (qd_rk43_start and
// qd_rk43_resume clear them), so a flag the commit's refresh solve raised
// stays set until the next attempt's check or the call's last check reads
// it.
static int step_begin(qd_solver *s) {
    s->it = s->it + 1;
    return QD_OK;
}

// stages 2..6 and the error estimate of one attempt, and the copies of the
// error and of the solve state the host will read
static int attempt_enqueue(qd_solver *s) {
    const double *c = rk_c();
    s->attempts++;
    if (s->t + s->dt > s->P.tmax) s->dt = s->P.tmax - s->t;
    for (int st = 2; st <= 6; st++) QD_TRY(stage(s, st, c[st]));
    // the attempt's report: written by the error kernel into the pinned
    // host copies where the device can address them, else three copies
    const bool mapped = s->dh_scal && s->dh_solve && s->dh_status;
    QD_TRY(launch_error(s, mapped));
    if (mapped) return QD_OK;
    QD_CUDA(cudaMemcpyAsync(s->h_scal + 2, s->d_scal + 2, sizeof(double), cudaMemcpyDeviceToHost,
                            s->stream));
    QD_CUDA(cudaMemcpyAsync(s->h_solve, s->d_solve, sizeof(SolveState), cudaMemcpyDeviceToHost, s->stream));
    QD_CUDA(cudaMemcpyAsync(s->h_status, s->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
    return QD_OK;
}

// the attempt's one synchronisation; *retry: reduce dt and attempt again.
// A failed solve or Newton solve ends the step at the attempt that met it
// (the reference exits in NRsearch at the first NaN, fault.cpp:211-225).
static int attempt_finish(qd_solver *s, int attemptCount, double *totErr, int *retry) {
    QD_CUDA(cudaStreamSynchronize(s->stream));
    // a Newton failure first: its NaN reaches the next stage's boundary data
    // and makes that solve fail too
    QD_TRY(status_flag_error(*s->h_status));
    QD_TRY(solve_flag_error(*s->h_solve));
    warm_start_standby_update(s, s->h_solve->need_max);
    *totErr = s->h_scal[2];
    *retry = 0;
    if (*totErr < s->P.totTol) return QD_OK;
    s->dt = step_size(s->it, s->dt, s->P, *totErr, s->errA);
    if (s->P.mindt == s->dt) return QD_OK;
    *retry = attemptCount < 100;
    return QD_OK;
}

static int commit_enqueue(qd_solver *s) {
    s->t = s->t + s->dt;
    return stage(s, 1, 0.0, true);   // the commit (:1606-1614) in the refresh stage's launch (:1615-1619)
}

// the host's side of a commit; check: wait for the refresh and read the
// failure flags now (otherwise the next attempt's check, or the last check
// of the call, reads them: one host wait fewer per step)
static int commit_finish(qd_solver *s, double totErr, bool check) {
    const double newDeltaT = (totErr != 0.0) ? step_size(s->it, s->dt, s->P, totErr, s->errA) : s->dt;
    s->errA[1] = s->errA[0];
    s->errA[0] = totErr;
    s->dt = newDeltaT;
    s->steps++;
    return check ? check_status(s) : QD_OK;
}

static int rk_step(qd_solver *s, bool check) {
    QD_TRY(step_begin(s));
    double totErr = 0.0;
    int retry = 1;
    for (int attemptCount = 1; retry; attemptCount++) {
        QD_TRY(attempt_enqueue(s));
        QD_TRY(attempt_finish(s, attemptCount, &totErr, &retry));
    }
    QD_TRY(commit_enqueue(s));
    return commit_finish(s, totErr, check);
}

static bool can_step(const qd_solver *s) { return s->it < s->P.maxNumSteps && s->t < s->P.tmax; }

}  // namespace qd

using namespace qd;

extern "C" {

const char *qd_version(void) { return "qdeq-gb300 1 (sm_103a)"; }
const char *qd_last_error(void) { return g_err; }

void qd_default_options(qd_mg_options *o) {
    if (!o) return;
    o->n_levels = 6;
    o->nu_pre = 32;
    o->nu_post = 32;
    o->nu_coarse = 32;
    o->tol_mode = QD_TOL_ABS;
    o->tol = 1e-9;
    o->max_cycles = 0;
    o->precision = QD_PREC_FP64;
    o->surface_prolong = 0;
    o->coarse_solve = 0;
}

int qd_solver_create(int ni, int nk, double dh, const double *mu_equi, const double *mu_node,
                     const qd_mg_options *opt, qd_solver **out) {
    return qd_solver_create_mapped(ni, nk, dh, mu_equi, mu_node, nullptr, opt, out);
}

int qd_solver_create_mapped(int ni, int nk, double dh, const double *mu_equi, const double *mu_node,
                            const double *jrow, const qd_mg_options *opt, qd_solver **out) {
    if (!out || !mu_equi || !mu_node || ni < 3 || nk < 3 || !(dh > 0.0)) {
        set_error("qd_solver_create: bad arguments");
        return QD_ERR_ARG;
    }
    if (jrow)
        for (int r = 0; r < 2 * (nk + 2) - 1; r++)
            if (!(jrow[r] > 0.0) || !std::isfinite(jrow[r])) {
                set_error("qd_solver_create_mapped: the depth metric must be positive and finite (row %d)", r);
                return QD_ERR_ARG;
            }
    *out = nullptr;
    QD_TRY(check_opts(opt));
    qd_solver *s = new qd_solver();
    memset((void *)s, 0, sizeof(*s));
    s->net_cost = kNetCostCycles;   // the measured gate: run the network where a guess
    s->net_ratio = -kNetCostCycles; // needs more than 1 + cost V-cycles
    s->ni = ni; s->nk = nk; s->nx = ni + 2; s->nz = nk + 2; s->dh = dh;
    s->opt = *opt;
    int rc = QD_OK;
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&s->d_scal, 8 * sizeof(double)) != cudaSuccess ||
        cudaMallocHost(&s->h_scal, 8 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&s->d_status, sizeof(DevStatus)) != cudaSuccess ||
        cudaMallocHost(&s->h_status, sizeof(DevStatus)) != cudaSuccess ||
        cudaMalloc(&s->d_solve, sizeof(SolveState)) != cudaSuccess ||
        cudaMemset(s->d_solve, 0, sizeof(SolveState)) != cudaSuccess ||
        cudaMallocHost(&s->h_solve, sizeof(SolveState)) != cudaSuccess) {
        set_error("qd_solver_create: CUDA set-up failed: %s", cudaGetErrorString(cudaGetLastError()));
        qd_solver_destroy(s);
        return QD_ERR_CUDA;
    }
    {   // device addresses of the pinned host copies (the error kernel's
        // attempt report); none where the device cannot address them
        void *a = nullptr, *b = nullptr, *c = nullptr;
        if (cudaHostGetDevicePointer(&a, s->h_scal, 0) == cudaSuccess &&
            cudaHostGetDevicePointer(&b, s->h_solve, 0) == cudaSuccess &&
            cudaHostGetDevicePointer(&c, s->h_status, 0) == cudaSuccess) {
            s->dh_scal = static_cast<double *>(a);
            s->dh_solve = static_cast<SolveState *>(b);
            s->dh_status = static_cast<DevStatus *>(c);
        } else {
            (void)cudaGetLastError();
        }
    }
    rc = mg_alloc(s, mu_equi, jrow);
    if (rc == QD_OK) rc = fault_alloc(s);
    if (rc == QD_OK) {
        std::vector<double> mu0(s->nz, 0.0);
        for (int k = 0; k < s->nz; k++) mu0[k] = mu_node[1 + (long)k * s->nx];   // fault.cpp:151-153
        if (cudaMemcpy(s->F.mu0, mu0.data(), s->nz * sizeof(double), cudaMemcpyHostToDevice) !=
            cudaSuccess)
            rc = QD_ERR_CUDA;
    }
    if (rc == QD_OK) rc = reset_status(s);
    if (rc == QD_OK && cudaStreamSynchronize(s->stream) != cudaSuccess) rc = QD_ERR_CUDA;
    if (rc != QD_OK) {
        qd_solver_destroy(s);
        return rc;
    }
    *out = s;
    return QD_OK;
}

int qd_solver_destroy(qd_solver *s) {
    if (!s) return QD_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    warm_start_detach(s);            // the network outlives the solver
    history_free(s);
    snapshot_free(s);                // waits for a snapshot still being written
    cudaFree(s->io_dev);
    cudaFreeHost(s->io_host);
    mg_free(s);
    fault_free(s);
    solve_graph_free(s);
    cudaFree(s->d_solve);
    cudaFreeHost(s->h_solve);
    cudaFree(s->d_scal);
    cudaFreeHost(s->h_scal);
    cudaFree(s->d_status);
    cudaFreeHost(s->h_status);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return QD_OK;
}

int qd_solver_set_options(qd_solver *s, const qd_mg_options *opt) {
    if (!s) return QD_ERR_ARG;
    QD_TRY(check_opts(opt));
    if (opt->n_levels != s->opt.n_levels) {
        set_error("n_levels cannot change after creation");
        return QD_ERR_ARG;
    }
    s->opt = *opt;
    return QD_OK;
}

int qd_get_stats(qd_solver *s, qd_stats *st) {
    if (!s || !st) return QD_ERR_ARG;
    SolveState ss;
    QD_TRY(solve_state_read(s, &ss));
    st->solves = (long long)ss.total_solves; st->vcycles = (long long)ss.total_cycles;
    st->attempts = s->attempts;
    // host-issued kernels plus the kernels the solve graphs ran on the device
    st->steps = s->steps; st->kernel_launches = s->launches + (long long)ss.kernels;
    st->net_solves = (long long)ss.net_solves;
    st->net_cycles_needed = ss.net_cycles_needed;
    st->net_cycles_taken = ss.net_cycles_taken;
    st->smooth_corrections = (long long)ss.total_smooths;
    st->net_armed_solves = s->net_armed_solves;
    std::vector<int> it(s->nz);
    QD_CUDA(cudaMemcpy(it.data(), s->F.iters, s->nz * sizeof(int), cudaMemcpyDeviceToHost));
    long long sum = 0;
    for (int v : it) sum += v;
    st->newton_iters = sum;
    return QD_OK;
}

void *qd_solver_stream(qd_solver *s) { return s ? (void *)s->stream : nullptr; }

int qd_set_medium(int ni, int nk, const double *mu_node, double *mu_equi) {
    return set_medium_gpu(ni, nk, mu_node, mu_equi);
}

}  // extern "C"

namespace qd {

// Host transfers of u and of the fault state go through staging buffers,
// one contiguous copy each way: a 2-D copy of the pitched field moves one
// row per DMA descriptor, and five 8-KB vector copies cost five API calls;
// a kernel then places the data.  At 1025^2 an upload of u took 72 us as a
// 2-D copy against 54 us for the same bytes in one copy.
static int io_staging(qd_solver *s) {
    if (s->io_dev) return QD_OK;
    const size_t nd = (size_t)s->nz * s->nx + 5 * (size_t)s->nz;
    if (cudaMalloc(&s->io_dev, nd * sizeof(double)) != cudaSuccess ||
        cudaMallocHost(&s->io_host, 5 * (size_t)s->nz * sizeof(double)) != cudaSuccess) {
        (void)cudaGetLastError();
        cudaFree(s->io_dev);
        s->io_dev = nullptr;
        set_error("transfer staging: out of memory");
        return QD_ERR_NOMEM;
    }
    return QD_OK;
}

// the interior of the ghosted nz x nx array G (rows 1..nk, columns 1..ni,
// :669-677) into the pitched level-0 field
__global__ void k_u_from_ghosted(const double *G, double *u, int N, int K, int P, int nx) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (k < K) u[(long)j * P + k] = G[(long)(j + 1) * nx + k + 1];
}

// the pitched level-0 field into the ghosted array with extend_crew's ghost
// values (odeSolver.cpp:612-650): ghost columns 2 U[1] - U[2] and
// 2 U[ni] - U[ni-1] on every row, then ghost rows 0 and nk+1 copies of rows
// 2 and nk-1 (ghost columns included).  2a is exact, so the expression rounds
// as the host's does.
__global__ void k_u_to_ghosted(const double *u, double *G, int ni, int nk, int P) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
    const int nx = ni + 2;
    if (c >= nx) return;
    const int rr = r == 0 ? 2 : (r == nk + 1 ? nk - 1 : r);     // the row the value comes from
    const double *row = u + (long)(rr - 1) * P - 1;               // row[c]: ghosted column c
    double v;
    if (c == 0) v = 2.0 * row[1] - row[2];
    else if (c == ni + 1) v = 2.0 * row[ni] - row[ni - 1];
    else v = row[c];
    G[(long)r * nx + c] = v;
}

// up to five nz-vectors gathered into (get) or scattered from (put) the
// packed staging vector
struct Vec5 {
    double *p[5];
};
__global__ void k_vec5(Vec5 v, double *packed, int nz, int put) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, q = blockIdx.y;
    if (i >= nz || !v.p[q]) return;
    if (put) v.p[q][i] = packed[(long)q * nz + i];
    else packed[(long)q * nz + i] = v.p[q][i];
}

}  // namespace qd

extern "C" {

int qd_upload_u(qd_solver *s, const double *U) {
    if (!s || !U) return QD_ERR_ARG;
    QD_TRY(io_staging(s));
    const LevelDims &d = s->dims[0];
    QD_CUDA(cudaMemcpyAsync(s->io_dev, U, sizeof(double) * (size_t)s->nz * s->nx, cudaMemcpyHostToDevice,
                            s->stream));
    k_u_from_ghosted<<<dim3((d.K + 255) / 256, d.N), 256, 0, s->stream>>>(s->io_dev, s->L64[0].u, d.N, d.K, d.P,
                                                                          s->nx);
    QD_LAUNCH_CHECK(s);
    QD_CUDA(cudaStreamSynchronize(s->stream));
    return QD_OK;
}

int qd_download_u(qd_solver *s, double *U) {
    if (!s || !U) return QD_ERR_ARG;
    QD_TRY(io_staging(s));
    const LevelDims &d = s->dims[0];
    k_u_to_ghosted<<<dim3((s->nx + 255) / 256, s->nz), 256, 0, s->stream>>>(s->L64[0].u, s->io_dev, s->ni, s->nk,
                                                                             d.P);
    QD_LAUNCH_CHECK(s);
    QD_CUDA(cudaMemcpyAsync(U, s->io_dev, sizeof(double) * (size_t)s->nz * s->nx, cudaMemcpyDeviceToHost,
                            s->stream));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    return QD_OK;
}

int qd_ode_solve(qd_solver *s, int *cycles, double *rnorm, double *r0norm) {
    if (!s) return QD_ERR_ARG;
    s->net_standby = false;   // the standby is the RK loop's, decided per attempt
    return mg_solve(s, cycles, rnorm, r0norm);
}

int qd_ode_solve_host(qd_solver *s, double *U, int *cycles, double *rnorm) {
    QD_TRY(qd_upload_u(s, U));
    int rc = mg_solve(s, cycles, rnorm, nullptr);
    if (rc != QD_OK && rc != QD_ERR_NOT_CONVERGED) return rc;
    QD_TRY(qd_download_u(s, U));
    return rc;
}

int qd_mg_smooth(qd_solver *s, int nsweeps) {
    if (!s || nsweeps < 0) return QD_ERR_ARG;
    return mg_smooth(s, 0, nsweeps);
}

int qd_mg_vcycle(qd_solver *s) {
    if (!s) return QD_ERR_ARG;
    return mg_vcycle(s);
}

int qd_mg_residual_norm(qd_solver *s, double *rnorm) {
    if (!s || !rnorm) return QD_ERR_ARG;
    return mg_residual_norm(s, rnorm);
}

int qd_convert_f64_to_f32(const double *in, float *out, int n) {
    if (!in || !out || n < 0) {
        set_error("qd_convert_f64_to_f32: bad arguments");
        return QD_ERR_ARG;
    }
    if (n == 0) return QD_OK;
    return convert_f64_f32(in, out, n);
}

int qd_split_f64(const double *in, float *hi, float *lo, int n) {
    if (!in || !hi || !lo || n < 0) {
        set_error("qd_split_f64: bad arguments");
        return QD_ERR_ARG;
    }
    if (n == 0) return QD_OK;
    return convert_f64_f32(in, hi, n, lo);
}

int qd_mg_time_kernel(qd_solver *s, int kernel, int reps, double *us) {
    if (!s || !us) {
        set_error("qd_mg_time_kernel: bad arguments");
        return QD_ERR_ARG;
    }
    if (kernel == QD_KERNEL_RESIDUAL && s->opt.precision != QD_PREC_MIXED) {
        set_error("qd_mg_time_kernel: the FP64-to-FP32 residual runs only in mixed precision");
        return QD_ERR_ARG;
    }
    return time_kernel(s, kernel, reps, us);
}

int qd_probe_bounded_wait(qd_solver *s, int polls) {
    if (!s || polls < 1 || polls > (int)TMA_WAIT_LIMIT) {
        set_error("qd_probe_bounded_wait: bad arguments (polls %d)", polls);
        return QD_ERR_ARG;
    }
    QD_TRY(wait_probe(s, (unsigned)polls));
    return check_status(s);
}

int qd_fault_setup(qd_solver *s, const double *a, const double *b, const double *eta,
                   const double *Tau_n0, const double *SlipShift, const double *tau0, double f0,
                   double V0, double L, double Vini) {
    if (!s || !a || !b || !eta || !Tau_n0 || !SlipShift) {
        set_error("qd_fault_setup: null array");
        return QD_ERR_ARG;
    }
    const size_t n = s->nz * sizeof(double);
    FaultState &F = s->F;
    QD_CUDA(cudaMemcpy(F.a, a, n, cudaMemcpyHostToDevice));
    QD_CUDA(cudaMemcpy(F.b, b, n, cudaMemcpyHostToDevice));
    QD_CUDA(cudaMemcpy(F.eta, eta, n, cudaMemcpyHostToDevice));
    QD_CUDA(cudaMemcpy(F.Tn0, Tau_n0, n, cudaMemcpyHostToDevice));
    QD_CUDA(cudaMemcpy(F.SlipShift, SlipShift, n, cudaMemcpyHostToDevice));
    if (tau0) QD_CUDA(cudaMemcpy(F.tau0, tau0, n, cudaMemcpyHostToDevice));
    F.have_tau0 = tau0 != nullptr;
    F.f0 = f0; F.V0 = V0; F.L = L; F.Vini = Vini;
    s->fault_ready = 1;
    return QD_OK;
}

int qd_set_boundary(qd_solver *s, const double *slip, double t_elapsed, double ratio, double dt) {
    if (!s || !slip) return QD_ERR_ARG;
    if (!s->fault_ready) { set_error("qd_set_boundary: no fault set up"); return QD_ERR_STATE; }
    QD_CUDA(cudaMemcpyAsync(s->F.Slip, slip, s->nz * sizeof(double), cudaMemcpyHostToDevice,
                            s->stream));
    const double t0 = s->t, dt0 = s->dt;
    s->t = t_elapsed;
    s->dt = dt;
    int rc = launch_stage_boundary(s, 1, ratio, false);
    s->t = t0;
    s->dt = dt0;
    QD_TRY(rc);
    QD_CUDA(cudaStreamSynchronize(s->stream));
    return QD_OK;
}

int qd_eval_stress_on_fault(qd_solver *s, double *Ts, double *Tn) {
    if (!s) return QD_ERR_ARG;
    if (!s->fault_ready) { set_error("qd_eval_stress_on_fault: no fault set up"); return QD_ERR_STATE; }
    QD_TRY(launch_stress(s));
    if (Ts) QD_CUDA(cudaMemcpyAsync(Ts, s->F.Ts, s->nz * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    if (Tn) QD_CUDA(cudaMemcpyAsync(Tn, s->F.Tn, s->nz * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    return QD_OK;
}

int qd_nrsearch(qd_solver *s, const double *Ts, const double *psi, double *V, int *iters) {
    if (!s || !Ts || !psi || !V) return QD_ERR_ARG;
    if (!s->fault_ready) { set_error("qd_nrsearch: no fault set up"); return QD_ERR_STATE; }
    const size_t n = s->nz * sizeof(double);
    // scratch: the stage-6 buffers are free outside qd_rk43_step
    double *dTs = s->F.kslip[6], *dpsi = s->F.kpsi[6], *dV = s->F.fV[6];
    QD_CUDA(cudaMemcpyAsync(dTs, Ts, n, cudaMemcpyHostToDevice, s->stream));
    QD_CUDA(cudaMemcpyAsync(dpsi, psi, n, cudaMemcpyHostToDevice, s->stream));
    QD_CUDA(cudaMemcpyAsync(dV, V, n, cudaMemcpyHostToDevice, s->stream));
    int *dit = nullptr;
    QD_CUDA(cudaMallocAsync(&dit, s->nz * sizeof(int), s->stream));
    QD_TRY(reset_status(s));
    QD_TRY(launch_newton(s, dTs, dpsi, dV, dit));
    QD_CUDA(cudaMemcpyAsync(V, dV, n, cudaMemcpyDeviceToHost, s->stream));
    if (iters) QD_CUDA(cudaMemcpyAsync(iters, dit, s->nz * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    QD_CUDA(cudaFreeAsync(dit, s->stream));
    return check_status(s);
}

int qd_cal_dpsi(qd_solver *s, const double *psi, const double *V, double *dpsi) {
    if (!s || !psi || !V || !dpsi) return QD_ERR_ARG;
    if (!s->fault_ready) { set_error("qd_cal_dpsi: no fault set up"); return QD_ERR_STATE; }
    const size_t n = s->nz * sizeof(double);
    double *dp = s->F.kpsi[6], *dV = s->F.fV[6], *dd = s->F.fdpsi[6];
    QD_CUDA(cudaMemcpyAsync(dp, psi, n, cudaMemcpyHostToDevice, s->stream));
    QD_CUDA(cudaMemcpyAsync(dV, V, n, cudaMemcpyHostToDevice, s->stream));
    QD_TRY(launch_dpsi(s, dp, dV, dd));
    QD_CUDA(cudaMemcpyAsync(dpsi, dd, n, cudaMemcpyDeviceToHost, s->stream));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    return QD_OK;
}

int qd_rk43_start(qd_solver *s, const qd_rk43_params *p, const double *Slip, const double *psi) {
    if (!s || !p || !Slip || !psi) return QD_ERR_ARG;
    if (!s->fault_ready) { set_error("qd_rk43_start: no fault set up"); return QD_ERR_STATE; }
    if (p->maxNumSteps == 0) { set_error("max number of steps == 0"); return QD_ERR_ARG; }  // :1357-1361
    s->P = *p;
    const size_t n = s->nz * sizeof(double);
    QD_CUDA(cudaMemcpy(s->F.Slip, Slip, n, cudaMemcpyHostToDevice));
    QD_CUDA(cudaMemcpy(s->F.psi, psi, n, cudaMemcpyHostToDevice));
    for (int st = 1; st <= 6; st++) {
        QD_CUDA(cudaMemset(s->F.fV[st], 0, n));
        QD_CUDA(cudaMemset(s->F.fdpsi[st], 0, n));
    }
    s->t = 0.0;
    s->it = 0;
    s->errA[0] = s->errA[1] = 0.0;
    history_reset(s);
    return rk_start(s);
}

int qd_rk43_resume(qd_solver *s, const qd_rk43_params *p, const double *Slip, const double *psi, double t,
                   double dt, double errA0, double errA1, int it) {
    if (!s || !p || !Slip || !psi || !(dt > 0.0) || it < 0) {
        set_error("qd_rk43_resume: bad arguments");
        return QD_ERR_ARG;
    }
    if (!s->fault_ready) { set_error("qd_rk43_resume: no fault set up"); return QD_ERR_STATE; }
    if (p->maxNumSteps == 0) { set_error("max number of steps == 0"); return QD_ERR_ARG; }
    s->P = *p;
    const size_t n = s->nz * sizeof(double);
    QD_CUDA(cudaMemcpy(s->F.Slip, Slip, n, cudaMemcpyHostToDevice));
    QD_CUDA(cudaMemcpy(s->F.psi, psi, n, cudaMemcpyHostToDevice));
    for (int st = 1; st <= 6; st++) {     // zero Newton seeds, as after a commit (:1605-1614)
        QD_CUDA(cudaMemset(s->F.fV[st], 0, n));
        QD_CUDA(cudaMemset(s->F.fdpsi[st], 0, n));
    }
    s->t = t;
    s->it = it;
    s->errA[0] = errA0;
    s->errA[1] = errA1;
    history_reset(s);
    QD_TRY(reset_status(s));
    QD_TRY(solve_state_clear_flag(s));
    s->dt = dt;
    QD_TRY(stage(s, 1, 0.0));     // the refresh solve and fault update of a commit (:1615-1619)
    QD_TRY(check_status(s));
    s->started = 1;
    return QD_OK;
}

int qd_ensemble_step(qd_solver **ss, int n, int nsteps, int *steps_done) {
    if (!ss || n < 1 || nsteps < 0) {
        set_error("qd_ensemble_step: bad arguments");
        return QD_ERR_ARG;
    }
    for (int i = 0; i < n; i++) {
        if (!ss[i]) { set_error("qd_ensemble_step: solver %d is NULL", i); return QD_ERR_ARG; }
        if (!ss[i]->started) { set_error("qd_ensemble_step: solver %d not started", i); return QD_ERR_STATE; }
        for (int j = 0; j < i; j++)
            if (ss[j] == ss[i]) { set_error("qd_ensemble_step: solver %d listed twice", i); return QD_ERR_ARG; }
        if (steps_done) steps_done[i] = 0;
    }
    std::vector<char> act(n), trying(n);
    std::vector<int> att(n);
    std::vector<double> err(n);
    for (int k = 0; k < nsteps; k++) {
        int nact = 0;
        for (int i = 0; i < n; i++) {
            act[i] = can_step(ss[i]);
            if (!act[i]) continue;
            nact++;
            QD_TRY(step_begin(ss[i]));
            trying[i] = 1;
            att[i] = 0;
        }
        if (!nact) break;
        for (int left = nact; left > 0;) {
            // every instance still trying enqueues its attempt before any waits
            for (int i = 0; i < n; i++)
                if (act[i] && trying[i]) {
                    att[i]++;
                    QD_TRY(attempt_enqueue(ss[i]));
                }
            for (int i = 0; i < n; i++)
                if (act[i] && trying[i]) {
                    int retry = 0;
                    QD_TRY(attempt_finish(ss[i], att[i], &err[i], &retry));
                    if (!retry) {
                        trying[i] = 0;
                        left--;
                    }
                }
        }
        for (int i = 0; i < n; i++)
            if (act[i]) QD_TRY(commit_enqueue(ss[i]));
        for (int i = 0; i < n; i++)
            if (act[i]) {
                QD_TRY(commit_finish(ss[i], err[i], false));
                if (steps_done) steps_done[i]++;
            }
    }
    for (int i = 0; i < n; i++) QD_TRY(check_status(ss[i]));   // the last refresh solves' flags
    return QD_OK;
}

int qd_rk43_step(qd_solver *s, int nsteps, int *steps_done) {
    if (!s || nsteps < 0) return QD_ERR_ARG;
    if (!s->started) { set_error("qd_rk43_step before qd_rk43_start"); return QD_ERR_STATE; }
    int done = 0;
    int rc = QD_OK;
    while (done < nsteps && s->it < s->P.maxNumSteps && s->t < s->P.tmax) {   // :1462
        rc = rk_step(s, false);
        if (rc != QD_OK) break;
        done++;
    }
    if (rc == QD_OK && done > 0) rc = check_status(s);   // the last refresh solve's flags
    if (steps_done) *steps_done = done;
    return rc;
}

int qd_rk43_step_host(qd_solver *s, int nsteps, double *Slip, double *psi, double *V, double *dpsi, double *Ts,
                      double *U, double *state4, int *it, int *steps_done) {
    if (!s || nsteps < 0 || !Slip || !psi || !V || !dpsi || !U || !state4 || !it) return QD_ERR_ARG;
    if (!s->fault_ready) { set_error("qd_rk43_step_host: no fault set up"); return QD_ERR_STATE; }
    QD_TRY(io_staging(s));
    QD_CUDA(cudaStreamSynchronize(s->stream));      // the pinned staging is free
    const LevelDims &d = s->dims[0];
    const size_t n = s->nz * sizeof(double);
    double *packed = s->io_dev + (size_t)s->nz * s->nx;
    // in: the state vectors packed into one copy, u in one copy, both placed by kernels
    const double *src[4] = {Slip, psi, V, dpsi};
    for (int q = 0; q < 4; q++) memcpy(s->io_host + (size_t)q * s->nz, src[q], n);
    QD_CUDA(cudaMemcpyAsync(packed, s->io_host, 4 * n, cudaMemcpyHostToDevice, s->stream));
    Vec5 vin = {{s->F.Slip, s->F.psi, s->F.fV[1], s->F.fdpsi[1], nullptr}};
    k_vec5<<<dim3((s->nz + 255) / 256, 5), 256, 0, s->stream>>>(vin, packed, s->nz, 1);
    QD_LAUNCH_CHECK(s);
    QD_CUDA(cudaMemcpyAsync(s->io_dev, U, sizeof(double) * (size_t)s->nz * s->nx, cudaMemcpyHostToDevice,
                            s->stream));
    k_u_from_ghosted<<<dim3((d.K + 255) / 256, d.N), 256, 0, s->stream>>>(s->io_dev, s->L64[0].u, d.N, d.K, d.P,
                                                                          s->nx);
    QD_LAUNCH_CHECK(s);
    s->t = state4[0]; s->dt = state4[1]; s->errA[0] = state4[2]; s->errA[1] = state4[3]; s->it = *it;
    s->started = 1;
    int done = 0;
    int rc = QD_OK;
    while (done < nsteps && s->it < s->P.maxNumSteps && s->t < s->P.tmax) {   // :1462
        rc = rk_step(s, false);
        if (rc != QD_OK) break;
        done++;
    }
    if (steps_done) *steps_done = done;
    if (rc != QD_OK) return rc;
    // the last refresh solve's flags, read with the results
    QD_CUDA(cudaMemcpyAsync(s->h_status, s->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
    QD_CUDA(cudaMemcpyAsync(s->h_solve, s->d_solve, sizeof(SolveState), cudaMemcpyDeviceToHost, s->stream));
    // out: the state vectors gathered into one copy, u with its ghost values in one copy
    Vec5 vout = {{s->F.Slip, s->F.psi, s->F.fV[1], s->F.fdpsi[1], Ts ? s->F.Ts : nullptr}};
    k_vec5<<<dim3((s->nz + 255) / 256, 5), 256, 0, s->stream>>>(vout, packed, s->nz, 0);
    QD_LAUNCH_CHECK(s);
    QD_CUDA(cudaMemcpyAsync(s->io_host, packed, (Ts ? 5 : 4) * n, cudaMemcpyDeviceToHost, s->stream));
    k_u_to_ghosted<<<dim3((s->nx + 255) / 256, s->nz), 256, 0, s->stream>>>(s->L64[0].u, s->io_dev, s->ni, s->nk,
                                                                             d.P);
    QD_LAUNCH_CHECK(s);
    QD_CUDA(cudaMemcpyAsync(U, s->io_dev, sizeof(double) * (size_t)s->nz * s->nx, cudaMemcpyDeviceToHost,
                            s->stream));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    double *dst[5] = {Slip, psi, V, dpsi, Ts};
    for (int q = 0; q < 5; q++)
        if (dst[q]) memcpy(dst[q], s->io_host + (size_t)q * s->nz, n);
    state4[0] = s->t; state4[1] = s->dt; state4[2] = s->errA[0]; state4[3] = s->errA[1];
    *it = s->it;
    if (done > 0) {
        QD_TRY(status_flag_error(*s->h_status));
        QD_TRY(solve_flag_error(*s->h_solve));
    }
    return QD_OK;
}

int qd_rk43_get_state(qd_solver *s, double *Slip, double *psi, double *V, double *Ts, double *dpsi) {
    if (!s) return QD_ERR_ARG;
    QD_TRY(io_staging(s));
    double *dst[5] = {Slip, psi, V, Ts, dpsi};
    Vec5 v;
    const double *src[5] = {s->F.Slip, s->F.psi, s->F.fV[1], s->F.Ts, s->F.fdpsi[1]};
    for (int q = 0; q < 5; q++) v.p[q] = dst[q] ? const_cast<double *>(src[q]) : nullptr;
    double *packed = s->io_dev + (size_t)s->nz * s->nx;
    k_vec5<<<dim3((s->nz + 255) / 256, 5), 256, 0, s->stream>>>(v, packed, s->nz, 0);
    QD_LAUNCH_CHECK(s);
    QD_CUDA(cudaMemcpyAsync(s->io_host, packed, 5 * s->nz * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    for (int q = 0; q < 5; q++)
        if (dst[q]) memcpy(dst[q], s->io_host + (size_t)q * s->nz, s->nz * sizeof(double));
    return QD_OK;
}

int qd_rk43_get_scalars(qd_solver *s, double *d4, int *it) {
    if (!s) return QD_ERR_ARG;
    if (d4) { d4[0] = s->t; d4[1] = s->dt; d4[2] = s->errA[0]; d4[3] = s->errA[1]; }
    if (it) *it = s->it;
    return QD_OK;
}

int qd_rk43_set_state(qd_solver *s, const double *Slip, const double *psi, const double *V,
                      const double *dpsi, double t, double dt, double errA0, double errA1, int it) {
    if (!s || !Slip || !psi || !V || !dpsi) return QD_ERR_ARG;
    QD_TRY(io_staging(s));
    // the pinned staging may still feed an earlier transfer on the stream
    QD_CUDA(cudaStreamSynchronize(s->stream));
    const size_t n = s->nz * sizeof(double);
    const double *src[4] = {Slip, psi, V, dpsi};
    for (int q = 0; q < 4; q++) memcpy(s->io_host + (size_t)q * s->nz, src[q], n);
    double *packed = s->io_dev + (size_t)s->nz * s->nx;
    QD_CUDA(cudaMemcpyAsync(packed, s->io_host, 4 * n, cudaMemcpyHostToDevice, s->stream));
    Vec5 v = {{s->F.Slip, s->F.psi, s->F.fV[1], s->F.fdpsi[1], nullptr}};
    k_vec5<<<dim3((s->nz + 255) / 256, 5), 256, 0, s->stream>>>(v, packed, s->nz, 1);
    QD_LAUNCH_CHECK(s);
    QD_CUDA(cudaStreamSynchronize(s->stream));
    s->t = t; s->dt = dt; s->errA[0] = errA0; s->errA[1] = errA1; s->it = it;
    s->started = 1;
    return QD_OK;
}

int qd_set_tail_sweeps(qd_solver *s, int n) {
    if (!s || n < 0 || n > 64) {
        set_error("qd_set_tail_sweeps: n must be 0..64");
        return QD_ERR_ARG;
    }
    s->tail_sweeps = n;
    return QD_OK;
}

int qd_set_smooth_correction(qd_solver *s, double ratio) {
    if (!s || !(ratio == 0.0 || (ratio > 1.0 && ratio <= 1e6))) {
        set_error("qd_set_smooth_correction: ratio must be 0 or in (1, 1e6]");
        return QD_ERR_ARG;
    }
    if (ratio > 0.0 && s->opt.precision != QD_PREC_MIXED) {
        set_error("qd_set_smooth_correction: the smoothing pass needs mixed precision");
        return QD_ERR_ARG;
    }
    s->smooth_ratio = ratio;
    return QD_OK;
}

int qd_set_newton_start(qd_solver *s, int mode) {
    if (!s || (mode != 0 && mode != 1)) {
        set_error("qd_set_newton_start: mode must be 0 or 1");
        return QD_ERR_ARG;
    }
    s->newton_start = mode;
    return QD_OK;
}

int qd_set_solution_history(qd_solver *s, int m) {
    if (!s) return QD_ERR_ARG;
    return history_set(s, m);
}

int qd_solution_history_fit(qd_solver *s, double *coef, int *nd) {
    if (!s || !coef || !nd) return QD_ERR_ARG;
    return history_last_fit(s, coef, nd);
}

}  // extern "C"
