/*
 * ref_wrap.cpp -- extern "C" entry points onto the reference's own host
 * functions, for generating and checking golden vectors.  TEST
 * INFRASTRUCTURE ONLY; built by `make ref` together with the reference's
 * fault.cpp / Alloc.cpp / odeSolver.cpp (compiled in place, unmodified).
 *
 * The reference passes its structs by value (functions.h:11-45); these
 * wrappers build them from plain arrays laid out as the reference allocates
 * them (nz-long fault vectors, ghosted nx*nz fields) and call the reference.
 */
#include "struct.h"
#include "functions.h"

#include <string.h>

static GRID make_grid(int ni, int nk, double dh) {
    /* ode_init(), odeSolver.cpp:24-38 */
    GRID g;
    memset(&g, 0, sizeof(g));
    g.dh = dh; g.ni = ni; g.nk = nk;
    g.nx = ni + 2 * LEND; g.nz = nk + 2 * LEND;
    g.nx1 = 1; g.nx2 = g.nx1 + g.nx - 1; g.nz1 = 1; g.nz2 = g.nz1 + g.nz - 1;
    g.ni1 = g.nx1 + LEND; g.ni2 = g.ni1 + g.ni - 1;
    g.nk1 = g.nz1 + LEND; g.nk2 = g.nk1 + g.nk - 1;
    g.i0 = g.ni1; g.it = 0;
    return g;
}

extern "C" {

void ref_eval_stress_on_fault(int ni, int nk, double dh, double *U, double *mu_node,
                              double *Tau_n0, double *Ts, double *Tn) {
    GRID g = make_grid(ni, nk, dh);
    DISPLACEMENT d; d.Uy = U;
    PARAMS p; memset(&p, 0, sizeof(p));
    FAULT f; memset(&f, 0, sizeof(f));
    f.Ts = Ts; f.Tn = Tn; f.Tau_n0 = Tau_n0;
    MEDIUM m; memset(&m, 0, sizeof(m));
    m.mu = mu_node;
    eval_stress_on_fault(&g, d, &p, f, m);
}

void ref_nrsearch(int nk, double *Ts, double *Tn, double *a, double *eta, double *psi,
                  double V0, double *V) {
    GRID g = make_grid(3, nk, 1.0);
    FAULT f; memset(&f, 0, sizeof(f));
    f.Ts = Ts; f.Tn = Tn;
    RATE_STATE_LAW r; memset(&r, 0, sizeof(r));
    r.a = a; r.eta = eta; r.V0 = &V0;
    VARIABLE y; y.Slip = 0; y.psi = psi;
    Runge_Kutta rk; rk.V_f = V; rk.dpsi = 0;
    NRsearch(&g, f, r, y, rk);
}

void ref_cal_dpsi(int nk, double *psi, double *b, double *V, double f0, double V0,
                  double L, double *dpsi) {
    GRID g = make_grid(3, nk, 1.0);
    RATE_STATE_LAW r; memset(&r, 0, sizeof(r));
    r.b = b; r.f0 = &f0; r.V0 = &V0; r.L = &L;
    FAULT f; memset(&f, 0, sizeof(f));
    VARIABLE y; y.Slip = 0; y.psi = psi;
    Runge_Kutta rk; rk.V_f = V; rk.dpsi = dpsi;
    cal_dpsi(&g, r, f, y, rk);
}

double ref_compute_error(int nk, double *slip3, double *psi3, double *slip4, double *psi4) {
    GRID g = make_grid(3, nk, 1.0);
    VARIABLE y3; y3.Slip = slip3; y3.psi = psi3;
    VARIABLE y4; y4.Slip = slip4; y4.psi = psi4;
    return computeError(&g, y3, y4);
}

double ref_compute_step_size(int it, double dt, double mindt, double maxdt, double totErr,
                             double totTol, double *errA) {
    GRID g = make_grid(3, 3, 1.0);
    g.it = it;
    PARAMS p; memset(&p, 0, sizeof(p));
    p.dt = dt; p.mindt = mindt; p.maxdt = maxdt;
    return computeStepSize(&g, &p, totErr, totTol, errA);
}

void ref_set_boundary(int ni, int nk, double *U, double *slip, double *slip_shift,
                      double vini, double t, double ratio, double dt) {
    GRID g = make_grid(ni, nk, 1.0);
    DISPLACEMENT d; d.Uy = U;
    FAULT f; memset(&f, 0, sizeof(f));
    f.SlipShift = slip_shift;
    RATE_STATE_LAW r; memset(&r, 0, sizeof(r));
    r.Vini = &vini;
    VARIABLE y; y.Slip = slip; y.psi = 0;
    PARAMS p; memset(&p, 0, sizeof(p));
    p.t_elapsed = t; p.dt = dt;
    setBoundary(&g, d, f, r, y, &p, ratio);
}

void ref_extend_crew(int ni, int nk, double *U) {
    GRID g = make_grid(ni, nk, 1.0);
    DISPLACEMENT d; d.Uy = U;
    extend_crew(&g, d);
}

double ref_interp_2d(double *z12, double xi, double yi) {
    double x[3] = {-1.0, 0.0, 1.0};
    double y[4] = {-1.5, -0.5, 0.5, 1.5};
    double z[3][4];
    memcpy(z, z12, sizeof(z));
    return interp_2d(x, y, z, 3, 4, xi, yi);
}

double ref_interp2_2d(double *z12, double xi, double yi) {
    double x[4] = {-1.5, -0.5, 0.5, 1.5};
    double y[3] = {-1.0, 0.0, 1.0};
    double z[4][3];
    memcpy(z, z12, sizeof(z));
    return interp2_2d(x, y, z, 4, 3, xi, yi);
}

}  /* extern "C" */
