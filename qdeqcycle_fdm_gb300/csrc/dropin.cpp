// dropin.cpp -- the reference's hot-path functions (functions.h:11-45) with
// their signatures and struct.h types, over the C ABI.  RK43 keeps the
// reference's observable behaviour: the start solve, one printed line per
// accepted step and the snapshot records every it_save_jump steps.
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <string>
#include <vector>

#include "../../include/qdeq_functions.h"

namespace {

struct DropinConfig {
    qd_mg_options opt;
    const double *tau0 = nullptr;
    std::string outdir = "output";
    std::string tag = "qdeq";
    bool init = false;
};

DropinConfig &cfg() {
    static DropinConfig c;
    if (!c.init) {
        qd_default_options(&c.opt);
        c.init = true;
    }
    return c;
}

qd_solver *g_bound = nullptr;

bool ok(int rc, const char *what) {
    if (rc == QD_OK) return true;
    fprintf(stderr, "qdeq: %s failed (%d): %s\n", what, rc, qd_last_error());
    return false;
}

// snapshot record of odeSolver.cpp:1442-1456 (first) and :1638-1652
void write_record(const std::string &dir, int n, double t, double dt, int nx, int nz, const double *V,
                  const double *Slip, const double *Ts, const double *psi, const double *U,
                  const double *Tn, const double *a, const double *b) {
    mkdir(dir.c_str(), 0755);
    char name[1024];
    snprintf(name, sizeof(name), "%s/output_fault_%d.bin", dir.c_str(), n);
    FILE *fp = fopen(name, "wb");
    if (!fp) {
        fprintf(stderr, "qdeq: cannot write %s\n", name);
        return;
    }
    fwrite(&t, sizeof(double), 1, fp);
    fwrite(V, sizeof(double), nz, fp);
    fwrite(Slip, sizeof(double), nz, fp);
    fwrite(Ts, sizeof(double), nz, fp);
    fwrite(psi, sizeof(double), nz, fp);
    if (U) {
        fwrite(U, sizeof(double), (size_t)nx * nz, fp);
        fwrite(Tn, sizeof(double), nz, fp);
        fwrite(a, sizeof(double), nz, fp);
        fwrite(b, sizeof(double), nz, fp);
    }
    fwrite(&dt, sizeof(double), 1, fp);
    fclose(fp);
}

// maxval (fault.cpp:22-52) over the fault nodes nk1-1 .. nk2-1
double maxval(const double *v, int nk) {
    double m = v[1];
    for (int k = 2; k <= nk; k++)
        if (m < v[k]) m = v[k];
    return m;
}

}  // namespace

// tau0 is borrowed: the caller keeps its nz doubles alive until RK43 returns
extern "C" void qd_dropin_configure(const qd_mg_options *opt, const double *tau0,
                                    const char *outdir, const char *tag) {
    DropinConfig &c = cfg();
    if (opt) c.opt = *opt;
    if (tau0) c.tau0 = tau0;
    if (outdir) c.outdir = outdir;
    if (tag) c.tag = tag;
}

extern "C" void qd_dropin_bind(qd_solver *s) { g_bound = s; }

// RK43, odeSolver.cpp:1277-1674, on the GPU.
void RK43(int method, GRID *grid, PARAMS *params, DISPLACEMENT U, FAULT fault, MEDIUM medium,
          RATE_STATE_LAW RSL) {
    (void)method;
    DropinConfig &c = cfg();
    const int ni = grid->ni, nk = grid->nk, nx = grid->nx, nz = grid->nz;
    if (params->maxNumSteps == 0) {                                       // :1357-1361
        printf("ERROR: max number of steps == 0\n");
        return;
    }
    const double *tau0 = c.tau0;
    qd_solver *s = nullptr;
    if (!ok(qd_solver_create(ni, nk, grid->dh, medium.mu_equi, medium.mu, &c.opt, &s), "solver"))
        return;
    bool good = ok(qd_fault_setup(s, RSL.a, RSL.b, RSL.eta, fault.Tau_n0, fault.SlipShift, tau0,
                                  RSL.f0[0], RSL.V0[0], RSL.L[0], RSL.Vini[0]), "fault set-up") &&
                ok(qd_upload_u(s, U.Uy), "upload u");
    qd_rk43_params p = {params->tmax, params->ini_dt, params->mindt, params->maxdt, params->totTol,
                        params->maxNumSteps};
    std::vector<double> V(nz), dpsi(nz);
    good = good && ok(qd_rk43_start(s, &p, fault.Slip, RSL.psi), "RK43 start");
    if (good) {
        double d4[4];
        int it = 0;
        qd_rk43_get_state(s, fault.Slip, RSL.psi, V.data(), fault.Ts, dpsi.data());
        qd_rk43_get_scalars(s, d4, &it);
        for (int k = 1; k <= nk; k++) fault.Tn[k] = fault.Tau_n0[k];
        qd_download_u(s, U.Uy);
        params->dt = d4[1];
        printf("%s it=%d, dt=%.15lf, V_max=%.15e, Ts_max=%.15lf \n", c.tag.c_str(), grid->it,
               params->dt, maxval(V.data(), nk), maxval(fault.Ts, nk));
        write_record(c.outdir, 0, params->t_elapsed, params->dt, nx, nz, V.data(), fault.Slip,
                     fault.Ts, RSL.psi, U.Uy, fault.Tn, RSL.a, RSL.b);
        params->it_save = params->it_save + 1;
        while (grid->it < params->maxNumSteps && params->t_elapsed < params->tmax) {   // :1462
            int done = 0;
            if (!ok(qd_rk43_step(s, 1, &done), "RK43 step") || done == 0) break;
            qd_rk43_get_state(s, fault.Slip, RSL.psi, V.data(), fault.Ts, dpsi.data());
            qd_rk43_get_scalars(s, d4, &it);
            params->t_elapsed = d4[0];
            params->dt = d4[1];
            grid->it = it;
            printf("%s it=%d, dt=%.15lf, V_max=%.15e, Ts_max=%.15lf \n", c.tag.c_str(), grid->it,
                   params->dt, maxval(V.data(), nk), maxval(fault.Ts, nk));
            if (params->it_save_jump > 0 && grid->it % params->it_save_jump == 0) {
                write_record(c.outdir, params->it_save, params->t_elapsed, params->dt, nx, nz,
                             V.data(), fault.Slip, fault.Ts, RSL.psi, nullptr, nullptr, nullptr,
                             nullptr);
                params->it_save = params->it_save + 1;
            }
        }
        qd_download_u(s, U.Uy);
        for (int k = 0; k < nz; k++) {
            fault.V_f[k] = V[k];
            RSL.dpsi[k] = dpsi[k];
        }
    }
    qd_solver_destroy(s);
}

void ode_solve(int method, GRID *grid, DISPLACEMENT U, qd_solver *solver) {
    (void)method;
    (void)grid;
    qd_solver *s = solver ? solver : g_bound;
    if (!s) {
        fprintf(stderr, "qdeq: ode_solve without a solver\n");
        return;
    }
    int cycles = 0;
    double rn = 0.0;
    ok(qd_ode_solve_host(s, U.Uy, &cycles, &rn), "ode_solve");
}

// extend_crew, odeSolver.cpp:612-650
void extend_crew(GRID *grid, DISPLACEMENT U) {
    const int nx = grid->nx;
    for (int k = grid->nz1 - 1; k < grid->nz2; k++)
        for (int n = 1; n < LEND + 1; n++) {
            const long i1 = grid->ni1 - 1 + (long)k * nx, i2 = grid->ni2 - 1 + (long)k * nx;
            U.Uy[i1 - n] = 2.0 * U.Uy[i1] - U.Uy[i1 + n];
            U.Uy[i2 + n] = 2.0 * U.Uy[i2] - U.Uy[i2 - n];
        }
    for (int n = 1; n < LEND + 1; n++)
        for (int i = grid->nx1 - 1; i < grid->nx2; i++) {
            const long i1 = i + (long)(grid->nk1 - 1) * nx, i2 = i + (long)(grid->nk2 - 1) * nx;
            U.Uy[i1 - (long)n * nx] = U.Uy[i1 + (long)n * nx];
            U.Uy[i2 + (long)n * nx] = U.Uy[i2 - (long)n * nx];
        }
}

// setBoundary, odeSolver.cpp:1150-1188 (host arrays)
void setBoundary(GRID *grid, DISPLACEMENT U, FAULT fault, RATE_STATE_LAW RSL, VARIABLE y,
                 PARAMS *params, double ratio) {
    const int nx = grid->nx, nz = grid->nz, nk1 = grid->nk1, nk2 = grid->nk2;
    for (int k = nk1 - 1; k < nk2; k++) U.Uy[(long)k * nx + grid->i0 - 1] = 0.5 * y.Slip[k];
    for (int k = 0; k < nz; k++)
        U.Uy[(long)k * nx + grid->ni2 - 1] =
            0.50 * RSL.Vini[0] * (params->t_elapsed + ratio * params->dt) + fault.SlipShift[k];
    for (int k = 0; k < nx; k++) U.Uy[(long)(nk1 - 2) * nx + k] = U.Uy[(long)nk1 * nx + k];
    for (int k = 0; k < nx; k++) U.Uy[(long)nk2 * nx + k] = U.Uy[(long)(nk2 - 2) * nx + k];
}

// eval_stress_on_fault, fault.cpp:139-156, on the bound solver's device
void eval_stress_on_fault(GRID *grid, DISPLACEMENT U, PARAMS *params, FAULT fault, MEDIUM medium) {
    (void)grid;
    (void)params;
    (void)medium;
    if (!g_bound) {
        fprintf(stderr, "qdeq: eval_stress_on_fault without a bound solver\n");
        return;
    }
    if (ok(qd_upload_u(g_bound, U.Uy), "upload u"))
        ok(qd_eval_stress_on_fault(g_bound, fault.Ts, fault.Tn), "eval_stress_on_fault");
}

// NRsearch, fault.cpp:169-232, on the bound solver's device
void NRsearch(GRID *grid, FAULT fault, RATE_STATE_LAW RSL, VARIABLE y, Runge_Kutta rk4) {
    (void)grid;
    (void)RSL;
    if (!g_bound) {
        fprintf(stderr, "qdeq: NRsearch without a bound solver\n");
        return;
    }
    ok(qd_nrsearch(g_bound, fault.Ts, y.psi, rk4.V_f, nullptr), "NRsearch");
}

// cal_dpsi, odeSolver.cpp:1190-1206, on the bound solver's device
void cal_dpsi(GRID *grid, RATE_STATE_LAW RSL, FAULT fault, VARIABLE y, Runge_Kutta rk4) {
    (void)grid;
    (void)RSL;
    (void)fault;
    if (!g_bound) {
        fprintf(stderr, "qdeq: cal_dpsi without a bound solver\n");
        return;
    }
    ok(qd_cal_dpsi(g_bound, y.psi, rk4.V_f, rk4.dpsi), "cal_dpsi");
}

// computeError, odeSolver.cpp:1211-1238
double computeError(GRID *grid, VARIABLE y3, VARIABLE y4) {
    double err1 = 0.0, err2 = 0.0;
    for (int k = grid->nk1 - 1; k < grid->nk2; k++) {
        const double t1 = y3.Slip[k] - y4.Slip[k], t2 = y3.psi[k] - y4.psi[k];
        err1 = err1 + t1 * t1;
        err2 = err2 + t2 * t2;
    }
    err1 = sqrt(err1);
    err2 = sqrt(err2);
    return err1 / (sqrt((double)grid->nk) * 1.0) + err2 / (sqrt((double)grid->nk) * 1.0);
}

// computeStepSize, odeSolver.cpp:1241-1271; a zero in the error history
// takes the elementary controller (the reference's PID branch would return
// mindt or NaN there), as the library's RK43 does
double computeStepSize(GRID *grid, PARAMS *params, const double totErr, double totTol,
                       double errA[2]) {
    const double ord = 4.0, kappa = 0.9;
    const double alpha = 0.49 / ord, beta = 0.34 / ord, gamma = 0.1 / ord;
    double stepRatio;
    if (grid->it < 4 || errA[0] == 0.0 || errA[1] == 0.0)
        stepRatio = kappa * pow(totTol / totErr, 1.0 / (1.0 + ord));
    else
        stepRatio = kappa * pow(totTol / totErr, alpha) * pow(errA[0] / totTol, beta) *
                    pow(totTol / errA[1], gamma);
    double deltaT = stepRatio * params->dt;
    deltaT = (params->dt * 5.0 <= deltaT) ? params->dt * 5.0 : deltaT;
    deltaT = (params->maxdt <= deltaT) ? params->maxdt : deltaT;
    deltaT = (params->mindt >= deltaT) ? params->mindt : deltaT;
    return deltaT;
}

// SetMedium's homogenisation (odeSolver.cpp:337-589) of the caller's
// medium.mu into medium.mu_equi, on the GPU
void SetMedium(GRID grid, COORD coord, MEDIUM medium, STRUCTURE structure) {
    (void)coord;
    (void)structure;
    ok(qd_set_medium(grid.ni, grid.nk, medium.mu, medium.mu_equi), "SetMedium");
}
