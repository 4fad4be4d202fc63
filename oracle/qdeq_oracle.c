/*
 * qdeq_oracle.c -- CPU restatement of QDEqCycle_FDM's per-stage hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the GB300 kernels and
 * the timed CPU baseline ("port").  Only tests/, __graft_entry__.smoke()
 * and bench.py may load it; the product library never does.
 *
 * Each function restates the reference function cited beside it, keeping
 * its index arithmetic, branch structure and operation order.  It is built
 * with -ffp-contract=off, so every multiply and add rounds separately.
 * Loops the reference runs one thread per grid point are OpenMP loops here;
 * each writes disjoint elements, so the thread count never changes a result.
 * Reductions go through per-row partial sums in a fixed order.
 */
#include "qdeq_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define LEND 1                 /* struct.h:8 */
#define RELAX 1.00             /* odeSolver.cpp:2 relax_rbgs */
#define QMIN(a, b) (((a) <= (b)) ? (a) : (b))   /* header.h:33 */
#define QMAX(a, b) (((a) >= (b)) ? (a) : (b))   /* header.h:32 */

int qo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void qo_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ====================================================================== */
/* multigrid                                                              */
/* ====================================================================== */

/* Level tables: RK43's GPU initialisation, odeSolver.cpp:1384-1417. */
int qo_mg_init(qo_mg *m, int ni, int nk, double dh, const double *mu_equi,
               int n_levels, int nu_pre, int nu_post, int nu_coarse) {
    memset(m, 0, sizeof(*m));
    if (n_levels < 1 || n_levels > QO_MAXLEV) return -1;
    m->n_levels = n_levels;
    m->nu_pre = nu_pre;
    m->nu_post = nu_post;
    m->nu_coarse = nu_coarse;
    m->nx = ni + 2 * LEND;
    m->mu = mu_equi;
    m->mux = mu_equi;
    m->muz = mu_equi;
    int n = nk, k = ni;
    double h = dh;
    m->N[0] = n; m->K[0] = k; m->fc[0] = 1; m->DH[0] = dh;
    for (int i = 0; i < n_levels - 1; i++) {
        m->res[i] = (double *)calloc((size_t)n * k, sizeof(double));
        n = (n - 1) / 2 + 1;
        k = (k - 1) / 2 + 1;
        h *= 2;
        m->res2[i] = (double *)calloc((size_t)n * k, sizeof(double));
        m->err2[i] = (double *)calloc((size_t)n * k, sizeof(double));
        m->fc[i + 1] = 1 << (i + 1);
        m->N[i + 1] = n; m->K[i + 1] = k; m->DH[i + 1] = h;
    }
    m->delta = (double *)calloc((size_t)nk * ni, sizeof(double));
    m->rowsum = (double *)calloc((size_t)nk, sizeof(double));
    return 0;
}

/* A grid stretched in depth: the x-face moduli times J and the z-face
 * moduli over J, J = dz/dzeta given per staggered row of mu_equi (the
 * conservative mapped form J d/dx(mu du/dx) + d/dzeta((mu/J) du/dzeta) on
 * the uniform computational grid).  The reference's grid is uniform
 * (coord.cpp:18,27); this is the project's own discretisation. */
void qo_mg_set_metric(qo_mg *m, int nk, const double *jrow) {
    free(m->own_x); free(m->own_z);
    m->own_x = m->own_z = NULL;
    m->mux = m->muz = m->mu;
    if (!jrow) return;
    const long W = 2L * m->nx - 1, R = 2L * (nk + 2 * LEND) - 1;
    m->own_x = (double *)malloc((size_t)(W * R) * sizeof(double));
    m->own_z = (double *)malloc((size_t)(W * R) * sizeof(double));
    for (long r = 0; r < R; r++)
        for (long c = 0; c < W; c++) {
            m->own_x[r * W + c] = m->mu[r * W + c] * jrow[r];
            m->own_z[r * W + c] = m->mu[r * W + c] / jrow[r];
        }
    m->mux = m->own_x;
    m->muz = m->own_z;
}

void qo_mg_free(qo_mg *m) {
    free(m->own_x); free(m->own_z);
    for (int i = 0; i < QO_MAXLEV; i++) {
        free(m->res[i]); free(m->res2[i]); free(m->err2[i]);
    }
    free(m->delta);
    free(m->rowsum);
    memset(m, 0, sizeof(*m));
}

/* The four face-coefficient indices of node (j,k) on a level:
 * level 0, odeSolver.cpp:785-789; coarse levels, odeSolver.cpp:823-827.
 * i3 (coarse, j=0) and i4 (coarse, j=N-1) can fall outside the array; the
 * callers never read them there, as the reference does not. */
static inline void mu_index(const qo_mg *m, int level, int j, int k,
                            long *i1, long *i2, long *i3, long *i4) {
    const long W = 2L * m->nx - 1;
    if (level == 0) {
        *i1 = ((k + LEND) * 2 - 1) + ((long)(j + LEND) * 2) * W;
        *i2 = ((k + LEND) * 2 + 1) + ((long)(j + LEND) * 2) * W;
        *i3 = (k + LEND) * 2 + ((long)(j + LEND) * 2 - 1) * W;
        *i4 = (k + LEND) * 2 + ((long)(j + LEND) * 2 + 1) * W;
    } else {
        const int fc = m->fc[level];
        *i1 = ((k * 2 - 1) * fc / 2 + LEND) * 2 + ((long)(j * fc + LEND) * 2) * W;
        *i2 = ((k * 2 + 1) * fc / 2 + LEND) * 2 + ((long)(j * fc + LEND) * 2) * W;
        *i3 = (k * fc + LEND) * 2 + ((long)((j * 2 - 1) * fc / 2 + LEND) * 2) * W;
        *i4 = (k * fc + LEND) * 2 + ((long)((j * 2 + 1) * fc / 2 + LEND) * 2) * W;
    }
}

/* rbgs_kernel<phase>, odeSolver.cpp:757-861.  Colour test (i+j+k)%2 with
 * i = 0 (:781); interior columns 1..K-2, all rows (:1412-1414). */
void qo_rbgs(const qo_mg *m, double *u, const double *f, int level, int phase) {
    const int N = m->N[level], K = m->K[level];
    const double DH2 = m->DH[level] * m->DH[level];
    const double *mx = m->mux, *mz = m->muz;   /* x-face / z-face moduli */
#pragma omp parallel for schedule(static)
    for (int j = 0; j < N; j++) {
        const int kstart = ((j + 1) % 2 == phase) ? 1 : 2;
        for (int k = kstart; k < K - 1; k += 2) {
            long i1, i2, i3, i4;
            mu_index(m, level, j, k, &i1, &i2, &i3, &i4);
            const long c = (long)j * K + k;
            const double uW = u[c - 1], uE = u[c + 1], uc = u[c], fv = f[c];
            double val;
            if (j == 0) {
                const double nb = u[c + K];
                if (level == 0) {   /* :792-800 */
                    val = (RELAX / (mx[i1] + mx[i2] + mz[i3] + mz[i4])) *
                              (mx[i1] * uW + mx[i2] * uE + mz[i3] * nb + mz[i4] * nb - DH2 * fv) +
                          (1.00 - RELAX) * uc;
                } else {            /* :830-838 */
                    val = (RELAX / (mx[i1] + mx[i2] + mz[i4] + mz[i4])) *
                              (mx[i1] * uW + mx[i2] * uE + mz[i4] * nb + mz[i4] * nb - DH2 * fv) +
                          (1.00 - RELAX) * uc;
                }
            } else if (j == N - 1) {
                const double nb = u[c - K];
                if (level == 0) {   /* :801-809 */
                    val = (RELAX / (mx[i1] + mx[i2] + mz[i3] + mz[i4])) *
                              (mx[i1] * uW + mx[i2] * uE + mz[i3] * nb + mz[i4] * nb - DH2 * fv) +
                          (1.00 - RELAX) * uc;
                } else {            /* :839-847 */
                    val = (RELAX / (mx[i1] + mx[i2] + mz[i3] + mz[i3])) *
                              (mx[i1] * uW + mx[i2] * uE + mz[i3] * nb + mz[i3] * nb - DH2 * fv) +
                          (1.00 - RELAX) * uc;
                }
            } else {                /* :810-818, :848-856 */
                val = (RELAX / (mx[i1] + mx[i2] + mz[i3] + mz[i4])) *
                          (mx[i1] * uW + mx[i2] * uE + mz[i3] * u[c - K] + mz[i4] * u[c + K] - DH2 * fv) +
                      (1.00 - RELAX) * uc;
            }
            u[c] = val;
        }
    }
}

/* residual_kernel, odeSolver.cpp:863-951 (calcuDelta_dev, :1045-1099, is
 * the same arithmetic on level 0). */
void qo_residual(const qo_mg *m, double *r, const double *u, const double *f, int level) {
    const int N = m->N[level], K = m->K[level];
    const double DH2 = m->DH[level] * m->DH[level];
    const double *mx = m->mux, *mz = m->muz;   /* x-face / z-face moduli */
#pragma omp parallel for schedule(static)
    for (int j = 0; j < N; j++) {
        for (int k = 1; k < K - 1; k++) {
            long i1, i2, i3, i4;
            mu_index(m, level, j, k, &i1, &i2, &i3, &i4);
            const long c = (long)j * K + k;
            const double uW = u[c - 1], uE = u[c + 1], uc = u[c], fv = f[c];
            double val;
            if (j == 0) {
                const double nb = u[c + K];
                if (level == 0) {
                    val = fv - (mx[i1] * uW + mx[i2] * uE + mz[i3] * nb + mz[i4] * nb -
                                (mx[i1] + mx[i2] + mz[i3] + mz[i4]) * uc) / DH2;
                } else {
                    val = fv - (mx[i1] * uW + mx[i2] * uE + mz[i4] * nb + mz[i4] * nb -
                                (mx[i1] + mx[i2] + mz[i4] + mz[i4]) * uc) / DH2;
                }
            } else if (j == N - 1) {
                const double nb = u[c - K];
                if (level == 0) {
                    val = fv - (mx[i1] * uW + mx[i2] * uE + mz[i3] * nb + mz[i4] * nb -
                                (mx[i1] + mx[i2] + mz[i3] + mz[i4]) * uc) / DH2;
                } else {
                    val = fv - (mx[i1] * uW + mx[i2] * uE + mz[i3] * nb + mz[i3] * nb -
                                (mx[i1] + mx[i2] + mz[i3] + mz[i3]) * uc) / DH2;
                }
            } else {
                val = fv - (mx[i1] * uW + mx[i2] * uE + mz[i3] * u[c - K] + mz[i4] * u[c + K] -
                            (mx[i1] + mx[i2] + mz[i3] + mz[i4]) * uc) / DH2;
            }
            r[c] = val;
        }
    }
}

/* restriction_kernel, odeSolver.cpp:953-1015.  `level` is the coarse level. */
void qo_restriction(const qo_mg *m, double *r2, const double *r, double *e2, int level) {
    const int Nc = m->N[level], Kc = m->K[level], Kf = m->K[level - 1];
#define RF(jj, kk) r[(long)(jj) * Kf + (kk)]
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Nc; j++) {
        for (int k = 1; k < Kc - 1; k++) {
            const long c = (long)j * Kc + k;
            double val;
            if (j == 0) {
                val = 0.06250 * (4.0 * RF(2 * j, 2 * k) + 2.0 * RF(2 * j, 2 * k - 1) +
                                 2.0 * RF(2 * j, 2 * k + 1) + 2.0 * RF(2 * j + 1, 2 * k) +
                                 2.0 * RF(2 * j + 1, 2 * k) + RF(2 * j + 1, 2 * k - 1) +
                                 RF(2 * j + 1, 2 * k + 1) + RF(2 * j + 1, 2 * k - 1) +
                                 RF(2 * j + 1, 2 * k + 1));
            } else if (j == Nc - 1) {
                val = 0.06250 * (4.0 * RF(2 * j, 2 * k) + 2.0 * RF(2 * j, 2 * k - 1) +
                                 2.0 * RF(2 * j, 2 * k + 1) + 2.0 * RF(2 * j - 1, 2 * k) +
                                 2.0 * RF(2 * j - 1, 2 * k) + RF(2 * j - 1, 2 * k - 1) +
                                 RF(2 * j - 1, 2 * k + 1) + RF(2 * j - 1, 2 * k - 1) +
                                 RF(2 * j - 1, 2 * k + 1));
            } else {
                val = 0.06250 * (4.0 * RF(2 * j, 2 * k) + 2.0 * RF(2 * j, 2 * k - 1) +
                                 2.0 * RF(2 * j, 2 * k + 1) + 2.0 * RF(2 * j - 1, 2 * k) +
                                 2.0 * RF(2 * j + 1, 2 * k) + RF(2 * j - 1, 2 * k - 1) +
                                 RF(2 * j - 1, 2 * k + 1) + RF(2 * j + 1, 2 * k - 1) +
                                 RF(2 * j + 1, 2 * k + 1));
            }
            r2[c] = val;
            e2[c] = 0.0;
        }
    }
#undef RF
}

/* prolongate_kernel, odeSolver.cpp:1017-1043.  `level` is the coarse level.
 * Coarse rows 0..Nc-2 and columns 0..Kc-2 only, so the last fine row never
 * receives a correction (:1034).  With m->surface_prolong the last coarse row
 * also corrects its coincident fine row (the project's option; not in the
 * reference). */
void qo_prolongate(const qo_mg *m, double *u, const double *e2, int level) {
    const int Nc = m->N[level], Kc = m->K[level], Kf = m->K[level - 1];
#define UF(jj, kk) u[(long)(jj) * Kf + (kk)]
#define EC(jj, kk) e2[(long)(jj) * Kc + (kk)]
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Nc - 1; j++) {
        for (int k = 0; k < Kc - 1; k++) {
            UF(2 * j, 2 * k) += EC(j, k);
            UF(2 * j, 2 * k + 1) += 0.5 * (EC(j, k) + EC(j, k + 1));
            UF(2 * j + 1, 2 * k) += 0.5 * (EC(j, k) + EC(j + 1, k));
            UF(2 * j + 1, 2 * k + 1) += 0.25 * (EC(j, k) + EC(j, k + 1) + EC(j + 1, k) + EC(j + 1, k + 1));
        }
    }
    if (m->surface_prolong) {
        const int j = Nc - 1;
        for (int k = 0; k < Kc - 1; k++) {
            UF(2 * j, 2 * k) += EC(j, k);
            UF(2 * j, 2 * k + 1) += 0.5 * (EC(j, k) + EC(j, k + 1));
        }
    }
#undef UF
#undef EC
}

/* smooth(), odeSolver.cpp:741-755: red (phase 0) then black, nsweeps times. */
void qo_smooth(const qo_mg *m, double *u, const double *f, int level, int nsweeps) {
    for (int it = 0; it < nsweeps; it++) {
        qo_rbgs(m, u, f, level, 0);
        qo_rbgs(m, u, f, level, 1);
    }
}

/* The project's exact coarsest-level solve (not in the reference): the
 * equations the smoother relaxes at `level`, with the same face moduli,
 * mirrored rows and row quirks as qo_rbgs, solved by Gaussian elimination
 * with partial pivoting on the interior unknowns. */
static void qo_coarse_solve(const qo_mg *m, double *u, const double *f, int level) {
    const int N = m->N[level], K = m->K[level], KI = K - 2, n = N * KI;
    const double DH2 = m->DH[level] * m->DH[level];
    const double *mx = m->mux, *mz = m->muz;   /* x-face / z-face moduli */
    double *A = (double *)calloc((size_t)n * (n + 1), sizeof(double));
#define AA(r, c) A[(size_t)(r) * (n + 1) + (c)]
    for (int j = 0; j < N; j++)
        for (int k = 1; k <= KI; k++) {
            long i1, i2, i3, i4;
            mu_index(m, level, j, k, &i1, &i2, &i3, &i4);
            double mN, mS;
            if (j == 0) { mN = (level == 0) ? mz[i3] : mz[i4]; mS = mz[i4]; }
            else if (j == N - 1) { mN = mz[i3]; mS = (level == 0) ? mz[i4] : mz[i3]; }
            else { mN = mz[i3]; mS = mz[i4]; }
            const int row = j * KI + (k - 1);
            const int jn = (j == 0) ? 1 : j - 1, js = (j == N - 1) ? N - 2 : j + 1;
            AA(row, row) -= (mx[i1] + mx[i2] + mN + mS) / DH2;
            if (k - 1 >= 1) AA(row, row - 1) += mx[i1] / DH2;
            if (k + 1 <= KI) AA(row, row + 1) += mx[i2] / DH2;
            AA(row, jn * KI + (k - 1)) += mN / DH2;
            AA(row, js * KI + (k - 1)) += mS / DH2;
            AA(row, n) = f[(long)j * K + k];
        }
    for (int c = 0; c < n; c++) {
        int p = c;
        for (int r = c + 1; r < n; r++)
            if (fabs(AA(r, c)) > fabs(AA(p, c))) p = r;
        if (p != c)
            for (int q = 0; q <= n; q++) { const double t = AA(p, q); AA(p, q) = AA(c, q); AA(c, q) = t; }
        for (int r = c + 1; r < n; r++) {
            const double fr = AA(r, c) / AA(c, c);
            if (fr == 0.0) continue;
            for (int q = c; q <= n; q++) AA(r, q) -= fr * AA(c, q);
        }
    }
    for (int r = n - 1; r >= 0; r--) {
        double s = AA(r, n);
        for (int q = r + 1; q < n; q++) s -= AA(r, q) * AA(q, n);
        AA(r, n) = s / AA(r, r);
    }
    for (int j = 0; j < N; j++)
        for (int k = 1; k <= KI; k++) u[(long)j * K + k] = AA(j * KI + (k - 1), n);
#undef AA
    free(A);
}

/* vcycle(), odeSolver.cpp:1101-1147. */
void qo_vcycle(qo_mg *m, double *u, const double *f, int level) {
    if (level >= m->n_levels - 1) {
        if (m->coarse_solve)
            qo_coarse_solve(m, u, f, level);
        else
            qo_smooth(m, u, f, level, m->nu_coarse);
        return;
    }
    double *r = m->res[level], *r2 = m->res2[level], *e2 = m->err2[level];
    qo_smooth(m, u, f, level, m->nu_pre);
    qo_residual(m, r, u, f, level);
    qo_restriction(m, r2, r, e2, level + 1);
    qo_vcycle(m, e2, r2, level + 1);
    qo_prolongate(m, u, e2, level + 1);
    qo_smooth(m, u, f, level, m->nu_post);
}

/* The L2 norm cublasDnrm2 takes at odeSolver.cpp:694,700 (whole N*K buffer;
 * the boundary columns hold zeros).  Summed per row, then over rows in
 * order. */
double qo_norm2(qo_mg *m, const double *r, int level) {
    const int N = m->N[level], K = m->K[level];
#pragma omp parallel for schedule(static)
    for (int j = 0; j < N; j++) {
        double s = 0.0;
        for (int k = 0; k < K; k++) s += r[(long)j * K + k] * r[(long)j * K + k];
        m->rowsum[j] = s;
    }
    double s = 0.0;
    for (int j = 0; j < N; j++) s += m->rowsum[j];
    return sqrt(s);
}

double qo_r0_norm(qo_mg *m, const double *u, int level) {
    const int N = m->N[level], K = m->K[level];
    const size_t n = (size_t)N * K;
    double *u0 = (double *)calloc(n, sizeof(double));
    double *f0 = (double *)calloc(n, sizeof(double));
    double *r0 = (double *)calloc(n, sizeof(double));
    for (int j = 0; j < N; j++) {
        u0[(long)j * K] = u[(long)j * K];
        u0[(long)j * K + K - 1] = u[(long)j * K + K - 1];
    }
    qo_residual(m, r0, u0, f0, level);
    double v = qo_norm2(m, r0, level);
    free(u0); free(f0); free(r0);
    return v;
}

/* multigrid(), odeSolver.cpp:652-720 (the device part: :693-705). */
int qo_multigrid(qo_mg *m, double *u, const double *f, int tol_mode, double tol,
                 int max_cycles, double *rnorm, double *r0norm) {
    double thr = tol;
    if (tol_mode == 1) {
        const double r0 = qo_r0_norm(m, u, 0);
        /* zero boundary data: the solution is u = 0; fall back to absolute */
        thr = r0 > 0.0 ? tol * r0 : tol;
        if (r0norm) *r0norm = r0;
    } else if (r0norm) {
        *r0norm = 0.0;
    }
    qo_residual(m, m->delta, u, f, 0);
    double delta = qo_norm2(m, m->delta, 0);
    int it = 0;
    while (delta > thr) {
        if (max_cycles > 0 && it >= max_cycles) break;
        qo_vcycle(m, u, f, 0);
        qo_residual(m, m->delta, u, f, 0);
        delta = qo_norm2(m, m->delta, 0);
        it++;
    }
    if (rnorm) *rnorm = delta;
    return it;
}

/* ====================================================================== */
/* boundary and ghosts                                                    */
/* ====================================================================== */

/* extend_crew(), odeSolver.cpp:612-650 (nx1 = nz1 = 1, ni1 = nk1 = 2). */
void qo_extend_crew(int ni, int nk, double *U) {
    const int nx = ni + 2 * LEND, nz = nk + 2 * LEND;
    const int ni1 = 1 + LEND, ni2 = ni1 + ni - 1, nk1 = 1 + LEND, nk2 = nk1 + nk - 1;
    for (int k = 0; k < nz; k++) {
        for (int n = 1; n < LEND + 1; n++) {
            const long index1 = ni1 - 1 + (long)k * nx;
            const long index2 = ni2 - 1 + (long)k * nx;
            U[index1 - n] = 2.0 * U[index1] - U[index1 + n];
            U[index2 + n] = 2.0 * U[index2] - U[index2 - n];
        }
    }
    for (int n = 1; n < LEND + 1; n++) {
        for (int i = 0; i < nx; i++) {
            const long index1 = i + (long)(nk1 - 1) * nx;
            const long index2 = i + (long)(nk2 - 1) * nx;
            U[index1 - (long)n * nx] = U[index1 + (long)n * nx];
            U[index2 + (long)n * nx] = U[index2 - (long)n * nx];
        }
    }
}

/* setBoundary(), odeSolver.cpp:1150-1188. */
void qo_set_boundary(int ni, int nk, double *U, const double *slip,
                     const double *slip_shift, double vini, double t_elapsed,
                     double ratio, double dt) {
    const int nx = ni + 2 * LEND, nz = nk + 2 * LEND;
    const int ni1 = 1 + LEND, ni2 = ni1 + ni - 1, nk1 = 1 + LEND, nk2 = nk1 + nk - 1;
    const int i0 = ni1;
    for (int k = nk1 - 1; k < nk2; k++) U[(long)k * nx + i0 - 1] = 0.5 * slip[k];
    for (int k = 0; k < nz; k++)
        U[(long)k * nx + ni2 - 1] = 0.50 * vini * (t_elapsed + ratio * dt) + slip_shift[k];
    for (int k = 0; k < nx; k++) U[(long)(nk1 - 2) * nx + k] = U[(long)nk1 * nx + k];
    for (int k = 0; k < nx; k++) U[(long)nk2 * nx + k] = U[(long)(nk2 - 2) * nx + k];
}

/* The host pack/unpack around the device solve, odeSolver.cpp:669-677 and
 * :708-716. */
void qo_pack(int ni, int nk, const double *U, double *u) {
    const int nx = ni + 2 * LEND, K = ni;
    for (int j = 1; j <= nk; j++)
        for (int i = 1; i <= ni; i++) u[(i - 1) + (long)(j - 1) * K] = U[i + (long)j * nx];
}

void qo_unpack(int ni, int nk, const double *u, double *U) {
    const int nx = ni + 2 * LEND, K = ni;
    for (int j = 1; j <= nk; j++)
        for (int i = 1; i <= ni; i++) U[i + (long)j * nx] = u[(i - 1) + (long)(j - 1) * K];
}

/* ====================================================================== */
/* fault physics                                                          */
/* ====================================================================== */

/* eval_stress_on_fault() + partial1st(), fault.cpp:139-164. */
void qo_eval_stress_on_fault(int ni, int nk, double dh, const double *U,
                             const double *mu_node, const double *Tau_n0,
                             double *Ts, double *Tn) {
    const int nx = ni + 2 * LEND;
    const int i0 = 1 + LEND;
    for (int k = 1; k <= nk; k++) {
        const long index = i0 - 1 + (long)k * nx;
        const double du = (-24.0 / (17.0 * dh)) * U[index] + (59.0 / (34.0 * dh)) * U[index + 1] +
                          (-4.0 / (17.0 * dh)) * U[index + 2] + (-3.0 / (34.0 * dh)) * U[index + 3];
        Ts[k] = mu_node[index] * du * 1.0e3;
        Tn[k] = Tau_n0[k];
    }
}

/* NRsearch(), fault.cpp:169-232. */
int qo_nrsearch(int nk, const double *Ts, const double *Tn, const double *tau0,
                const double *a, const double *eta, const double *psi,
                double V0, double *V, int *iters) {
    int status = 0;
    for (int k = 1; k <= nk; k++) {
        int iter = 0;
        double var_old = 0.5 * V[k] / V0 * exp(psi[k] / a[k]);
        var_old = asinh(var_old);
        const double fa = a[k] * fabs(Tn[k]);
        const double fb = tau0 ? Ts[k] + tau0[k] : Ts[k];
        const int iter_max = 100000;
        double var_new = var_old;
        while (iter < iter_max) {
            const double fy = 2.0 * eta[k] * V0 * exp(-psi[k] / a[k]) * sinh(var_old) + fa * var_old - fb;
            const double df = 2.0 * eta[k] * V0 * exp(-psi[k] / a[k]) * cosh(var_old) + fa;
            const double d = -fy / (df + 1e-100);
            var_new = var_old + d;
            const double err = fabs(d) / (fabs(var_old) + 1e-100);
            iter = iter + 1;
            var_old = var_new;
            if (err < 1e-10) break;
            /* A NaN iterate stays NaN; the reference spins to iter_max here
             * and ends with the same NaN, so stop early. */
            if (isnan(var_new)) break;
        }
        if (iters) iters[k] = iter;
        const double friction_update = a[k] * var_new;
        /* fault.cpp:211-225: a NaN is retried once from the same seed (which
         * can only repeat it) and then ends the program. */
        if (isnan(friction_update)) {
            if (status == 0) status = -1 - k;
            continue;
        }
        V[k] = 2.0 * V0 * exp(-psi[k] / a[k]);
        V[k] = V[k] * sinh(var_new);
    }
    return status;
}

/* cal_dpsi(), odeSolver.cpp:1190-1206 (aging law). */
void qo_cal_dpsi(int nk, const double *psi, const double *b, const double *V,
                 double f0, double V0, double L, double *dpsi) {
    for (int k = 1; k <= nk; k++) {
        const double A = exp((f0 - psi[k]) / b[k]);
        dpsi[k] = 0.0;
        if (!isinf(A) && b[k] > 1e-3) dpsi[k] = (b[k] * V0 / L) * (A - V[k] / V0);
    }
}

/* computeError(), odeSolver.cpp:1211-1238. */
double qo_compute_error(int nk, const double *slip3, const double *psi3,
                        const double *slip4, const double *psi4) {
    double err1 = 0.0, err2 = 0.0;
    for (int k = 1; k <= nk; k++) {
        const double t1 = slip3[k] - slip4[k];
        const double t2 = psi3[k] - psi4[k];
        err1 = err1 + t1 * t1;
        err2 = err2 + t2 * t2;
    }
    err1 = sqrt(err1);
    err2 = sqrt(err2);
    return err1 / (sqrt((double)nk) * 1.0) + err2 / (sqrt((double)nk) * 1.0);
}

/* computeStepSize(), odeSolver.cpp:1241-1271 (PID controller). */
double qo_compute_step_size(int it, double dt, double mindt, double maxdt,
                            double totErr, double totTol, const double errA[2]) {
    const double ord = 4.0, kappa = 0.9;
    const double alpha = 0.49 / ord, beta = 0.34 / ord, gamma = 0.1 / ord;
    double stepRatio;
    if (it < 4)
        stepRatio = kappa * pow(totTol / totErr, 1.0 / (1.0 + ord));
    else
        stepRatio = kappa * pow(totTol / totErr, alpha) * pow(errA[0] / totTol, beta) *
                    pow(totTol / errA[1], gamma);
    double deltaT = stepRatio * dt;
    deltaT = QMIN(dt * 5.0, deltaT);
    deltaT = QMIN(maxdt, deltaT);
    deltaT = QMAX(mindt, deltaT);
    return deltaT;
}

/* The step-size controller as the RK43 driver calls it.  computeStepSize's
 * PID branch divides by errA[1] and multiplies by errA[0]^beta; an accepted
 * step whose error estimate was exactly zero (the two embedded solutions
 * agree to the last bit, as happens on a perfectly steady fault) puts a zero
 * there, and the reference then yields dt = mindt or NaN.  With a zero in
 * the history this falls back to the elementary controller the reference
 * uses for its first steps (odeSolver.cpp:1254-1257). */
static double step_size_guarded(int it, double dt, double mindt, double maxdt,
                                double totErr, double totTol, const double errA[2]) {
    if (errA[0] == 0.0 || errA[1] == 0.0) it = 0;
    return qo_compute_step_size(it, dt, mindt, maxdt, totErr, totTol, errA);
}

/* ====================================================================== */
/* SetMedium homogenisation                                               */
/* ====================================================================== */

/* Lagrange basis of interp_2d()/interp2_2d(), odeSolver.cpp:134-268.  The
 * basis depends only on the stencil abscissae and the sample point, never on
 * the values, so it is computed once per sample with the reference's exact
 * loop; the per-edge sum then repeats the reference's summation order. */
static void lagrange_basis(const double *x, int n, double xi, double *L) {
    double xt[8], xb[8];
    for (int k = 0; k < n; k++) L[k] = 1.0;
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < n; k++) { xb[k] = x[k]; xb[k] = x[i] - xb[k]; }
        xb[i] = 1.0;
        for (int k = 0; k < n; k++) { xt[k] = x[k]; xt[k] = xi - xt[k]; }
        xt[i] = 1.0;
        for (int j = 0; j < n; j++) L[i] = L[i] * xt[j] / xb[j];
    }
}

/* interp_2d() / interp2_2d() for the two stencils SetMedium uses, through
 * the basis path above (exported so the basis path can be checked against
 * the reference's own interp functions). */
static double interp_sum(const double *z, int ni, int nj, const double *Lx, const double *Ly) {
    double zi = 0.0;
    for (int j = 0; j < nj; j++)
        for (int i = 0; i < ni; i++) zi = zi + Lx[i] * Ly[j] * z[i * nj + j];
    return zi;
}

double qo_interp_xedge(const double *z12, double xi, double yi) {
    static const double x[3] = {-1.0, 0.0, 1.0}, y[4] = {-1.5, -0.5, 0.5, 1.5};
    double Lx[4], Ly[4];
    lagrange_basis(x, 3, xi, Lx);
    lagrange_basis(y, 4, yi, Ly);
    return interp_sum(z12, 3, 4, Lx, Ly);
}

double qo_interp_zedge(const double *z12, double xi, double yi) {
    static const double x[4] = {-1.5, -0.5, 0.5, 1.5}, y[3] = {-1.0, 0.0, 1.0};
    double Lx[4], Ly[4];
    lagrange_basis(x, 4, xi, Lx);
    lagrange_basis(y, 3, yi, Ly);
    return interp_sum(z12, 4, 3, Lx, Ly);
}

#define NGRID 10
#define NSAMP ((2 * NGRID) * (2 * NGRID))

/* Harmonic mean of the NSAMP interpolated samples, odeSolver.cpp:442-460.
 * z is ni x nj, row-major (z[i*nj + j]); Lx[s] / Ly[s] are the bases. */
static double harmonic_edge(const double *z, int ni, int nj,
                            const double (*Lx)[4], const double (*Ly)[4]) {
    double mu0 = 0.0;
    int s = 0;
    for (int mj = -NGRID; mj <= NGRID; mj++) {
        if (mj == 0) continue;
        for (int mi = -NGRID; mi <= NGRID; mi++) {
            if (mi == 0) continue;
            const double zi = interp_sum(z, ni, nj, Lx[s], Ly[s]);
            mu0 = mu0 + 1.0 / zi;
            s++;
        }
    }
    return NSAMP / mu0;
}

/* SetMedium(), odeSolver.cpp:337-589 (the model set-up at :294-319 and the
 * file dumps are replaced by the caller's mu_node). */
void qo_set_medium(int ni, int nk, const double *mu_node, double *mu_half,
                   double *mu_equi) {
    const int nx = ni + 2 * LEND, nz = nk + 2 * LEND;
    const int ni1 = 1 + LEND, ni2 = ni1 + ni - 1, nk1 = 1 + LEND, nk2 = nk1 + nk - 1;
    const long W = 2L * nx - 1;
    const size_t n2 = (size_t)(2 * nx - 1) * (2 * nz - 1);
    memset(mu_half, 0, n2 * sizeof(double));
    memset(mu_equi, 0, n2 * sizeof(double));

    for (int k = nk1 - 1; k < nk2; k++)                    /* :337-346 */
        for (int i = ni1 - 1; i < ni2; i++) {
            const long index2 = i * 2 + ((long)k * 2) * W;
            mu_half[index2] = mu_node[i + (long)k * nx];
            mu_equi[index2] = mu_node[i + (long)k * nx];
        }
    for (int i = ni1 - 1; i < ni2; i++) {                  /* :347-353 */
        const long index = i * 2, index2 = i * 2 + ((long)(nk1 - 1) * 2) * W;
        mu_half[index] = mu_half[index2];
        mu_equi[index] = mu_half[index2];
    }
    for (int i = ni1 - 1; i < ni2; i++) {                  /* :354-360 */
        const long index = i * 2 + ((long)(nz - 1) * 2) * W;
        const long index2 = i * 2 + ((long)(nk2 - 1) * 2) * W;
        mu_half[index] = mu_half[index2];
        mu_equi[index] = mu_half[index2];
    }
    for (int k = 0; k < nz; k++) {                         /* :362-368 */
        const long index = ((long)k * 2) * W, index2 = (ni1 - 1) * 2 + ((long)k * 2) * W;
        mu_half[index] = mu_half[index2];
        mu_equi[index] = mu_half[index2];
    }
    for (int k = 0; k < nz; k++) {                         /* :370-376 */
        const long index = (nx - 1) * 2 + ((long)k * 2) * W;
        const long index2 = (ni2 - 1) * 2 + ((long)k * 2) * W;
        mu_half[index] = mu_half[index2];
        mu_equi[index] = mu_half[index2];
    }
    for (int k = 0; k < nz; k++)                           /* :381-392 */
        for (int i = ni1 - 1; i < ni2 - 1; i++) {
            const long index = i * 2 + ((long)k * 2) * W, index2 = (i + 1) * 2 + ((long)k * 2) * W;
            const long index3 = (i * 2 + 1) + ((long)k * 2) * W;
            mu_half[index3] = 0.50 * (mu_half[index] + mu_half[index2]);
        }
    for (int i = ni1 - 1; i < ni2; i++)                    /* :393-404 */
        for (int k = 0; k < nz - 1; k++) {
            const long index = i * 2 + ((long)k * 2) * W, index2 = i * 2 + ((long)(k + 1) * 2) * W;
            const long index3 = i * 2 + ((long)k * 2 + 1) * W;
            mu_half[index3] = 0.50 * (mu_half[index] + mu_half[index2]);
        }

    /* sample bases (:409-419, :454-456 and :498-500) */
    static const double x_index[3] = {-1.0, 0.0, 1.0};
    static const double y_index[4] = {-1.5, -0.5, 0.5, 1.5};
    static const double x_index2[4] = {-1.5, -0.5, 0.5, 1.5};
    static const double y_index2[3] = {-1.0, 0.0, 1.0};
    double (*LxA)[4] = calloc(NSAMP, sizeof(*LxA)), (*LyA)[4] = calloc(NSAMP, sizeof(*LyA));
    double (*LxB)[4] = calloc(NSAMP, sizeof(*LxB)), (*LyB)[4] = calloc(NSAMP, sizeof(*LyB));
    int s = 0;
    for (int mj = -NGRID; mj <= NGRID; mj++) {
        if (mj == 0) continue;
        for (int mi = -NGRID; mi <= NGRID; mi++) {
            if (mi == 0) continue;
            const double MI = mi / ((NGRID + 1.0) * 2.0), MJ = mj / ((NGRID + 1.0) * 2.0);
            lagrange_basis(x_index, 3, MI, LxA[s]);
            lagrange_basis(y_index, 4, MJ, LyA[s]);
            lagrange_basis(x_index2, 4, MI, LxB[s]);
            lagrange_basis(y_index2, 3, MJ, LyB[s]);
            s++;
        }
    }

#pragma omp parallel for schedule(static)
    for (int k = nk1 - 1; k < nk2; k++)                    /* x-edges :421-462 */
        for (int i = ni1; i < ni2; i++) {
            const long index = (i * 2 - 1) + ((long)k * 2) * W;
            const long index2 = (i - 2) * 2 + ((long)(k - 1) * 2) * W;
            const long index3 = (i - 2) * 2 + ((long)k * 2) * W;
            const long index4 = (i - 2) * 2 + ((long)(k + 1) * 2) * W;
            double z[12];
            for (int c = 0; c < 4; c++) {
                z[0 * 4 + c] = mu_half[index2 + 2 * c];
                z[1 * 4 + c] = mu_half[index3 + 2 * c];
                z[2 * 4 + c] = mu_half[index4 + 2 * c];
            }
            mu_equi[index] = harmonic_edge(z, 3, 4, (const double (*)[4])LxA, (const double (*)[4])LyA);
        }

#pragma omp parallel for schedule(static)
    for (int k = nk1; k < nk2; k++)                        /* z-edges :464-506 */
        for (int i = ni1; i < ni2 - 1; i++) {
            const long index = i * 2 + ((long)k * 2 - 1) * W;
            const long rows[4] = {(i - 1) * 2 + ((long)(k - 2) * 2) * W, (i - 1) * 2 + ((long)(k - 1) * 2) * W,
                                  (i - 1) * 2 + ((long)k * 2) * W, (i - 1) * 2 + ((long)(k + 1) * 2) * W};
            double z[12];
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 3; c++) z[r * 3 + c] = mu_half[rows[r] + 2 * c];
            mu_equi[index] = harmonic_edge(z, 4, 3, (const double (*)[4])LxB, (const double (*)[4])LyB);
        }

    for (int i = ni1; i < ni2 - 1; i++) {                  /* bottom-of-array z-edges :509-548 */
        const long index = i * 2 + ((long)(nk1 - 1) * 2 - 1) * W;
        const long rows[4] = {(i - 1) * 2, (i - 1) * 2, (i - 1) * 2 + ((long)(nk1 - 1) * 2) * W,
                              (i - 1) * 2 + ((long)nk1 * 2) * W};
        double z[12];
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 3; c++) z[r * 3 + c] = mu_half[rows[r] + 2 * c];
        mu_equi[index] = harmonic_edge(z, 4, 3, (const double (*)[4])LxB, (const double (*)[4])LyB);
    }
    for (int i = ni1; i < ni2 - 1; i++) {                  /* top-of-array z-edges :550-589 */
        const long index = i * 2 + ((long)nk2 * 2 - 1) * W;
        const long rows[4] = {(i - 1) * 2 + ((long)(nk2 - 2) * 2) * W, (i - 1) * 2 + ((long)(nk2 - 1) * 2) * W,
                              (i - 1) * 2 + ((long)nk2 * 2) * W, (i - 1) * 2 + ((long)nk2 * 2) * W};
        double z[12];
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 3; c++) z[r * 3 + c] = mu_half[rows[r] + 2 * c];
        mu_equi[index] = harmonic_edge(z, 4, 3, (const double (*)[4])LxB, (const double (*)[4])LyB);
    }
    free(LxA); free(LyA); free(LxB); free(LyB);
}

/* ====================================================================== */
/* RK43 driver                                                            */
/* ====================================================================== */

/* Explicit ARK4(3)6L tableau, odeSolver.cpp:1298-1334. */
static const double RK_C[7] = {0, 0, 1. / 2., 83. / 250., 31. / 50., 17. / 20., 1.};
static const double RK_B[7] = {0, 82889. / 524892., 0, 15625. / 83664., 69875. / 102672.,
                               -2260. / 8211., 1. / 4.};
static const double RK_HB[7] = {0, 4586570599. / 29645900160., 0, 178811875. / 945068544.,
                                814220225. / 1159782912., -3700637. / 11593932., 61727. / 225920.};
static const double RK_A[7][7] = {
    {0},
    {0},
    {0, 1. / 2.},
    {0, 13861. / 62500., 6889. / 62500.},
    {0, -116923316275. / 2393684061468., -2731218467317. / 15368042101831.,
     9408046702089. / 11113171139209.},
    {0, -451086348788. / 2902428689909., -2682348792572. / 7519795681897.,
     12662868775082. / 11960479115383., 3355817975965. / 11060851509271.},
    {0, 647845179188. / 3216320057751., 73281519250. / 8382639484533.,
     552539513391. / 3454668386233., 3354512671639. / 8306763924573., 4040. / 17871.},
};

struct qo_sim {
    int ni, nk, nx, nz;
    double dh;
    double tmax, t, dt, ini_dt, mindt, maxdt, totTol;
    int it, maxNumSteps;
    double errA[2];
    double f0, V0, L, Vini;
    double *a, *b, *eta, *Tau_n0, *Tn, *Ts, *Slip, *SlipShift, *psi, *tau0;
    int have_tau0;
    double *kslip[7], *kpsi[7], *fV[7], *fdpsi[7];
    double *y3s, *y3p, *y4s, *y4p;
    double *U, *u, *f, *mu_node;
    int *iters;
    qo_mg mg;
    int tol_mode, max_cycles;
    double tol;
    long long solves, vcycles, attempts, newton_iters;
    int status;
    qo_solve_hook hook;     /* replaces qo_multigrid in sim_solve when set */
    void *hook_ctx;
};

void qo_sim_set_solve_hook(qo_sim *s, qo_solve_hook fn, void *ctx) {
    s->hook = fn;
    s->hook_ctx = ctx;
}

static double *dz(size_t n) { return (double *)calloc(n, sizeof(double)); }

qo_sim *qo_sim_create(int ni, int nk, double dh, const double *mu_node,
                      const double *mu_equi, int n_levels, int nu_pre,
                      int nu_post, int nu_coarse, int tol_mode, double tol,
                      int max_cycles) {
    qo_sim *s = (qo_sim *)calloc(1, sizeof(qo_sim));
    s->ni = ni; s->nk = nk; s->nx = ni + 2; s->nz = nk + 2; s->dh = dh;
    const size_t nz = s->nz, nxz = (size_t)s->nx * s->nz;
    double **vecs[] = {&s->a, &s->b, &s->eta, &s->Tau_n0, &s->Tn, &s->Ts, &s->Slip,
                       &s->SlipShift, &s->psi, &s->tau0, &s->y3s, &s->y3p, &s->y4s, &s->y4p};
    for (size_t i = 0; i < sizeof(vecs) / sizeof(vecs[0]); i++) *vecs[i] = dz(nz);
    for (int st = 1; st <= 6; st++) {
        s->kslip[st] = dz(nz); s->kpsi[st] = dz(nz); s->fV[st] = dz(nz); s->fdpsi[st] = dz(nz);
    }
    s->iters = (int *)calloc(nz, sizeof(int));
    s->U = dz(nxz);
    s->mu_node = dz(nxz);
    memcpy(s->mu_node, mu_node, nxz * sizeof(double));
    s->u = dz((size_t)ni * nk);
    s->f = dz((size_t)ni * nk);
    qo_mg_init(&s->mg, ni, nk, dh, mu_equi, n_levels, nu_pre, nu_post, nu_coarse);
    s->tol_mode = tol_mode; s->tol = tol; s->max_cycles = max_cycles;
    return s;
}

void qo_sim_free(qo_sim *s) {
    if (!s) return;
    double *vecs[] = {s->a, s->b, s->eta, s->Tau_n0, s->Tn, s->Ts, s->Slip, s->SlipShift,
                      s->psi, s->tau0, s->y3s, s->y3p, s->y4s, s->y4p, s->U, s->mu_node, s->u, s->f};
    for (size_t i = 0; i < sizeof(vecs) / sizeof(vecs[0]); i++) free(vecs[i]);
    for (int st = 1; st <= 6; st++) {
        free(s->kslip[st]); free(s->kpsi[st]); free(s->fV[st]); free(s->fdpsi[st]);
    }
    free(s->iters);
    qo_mg_free(&s->mg);
    free(s);
}

void qo_sim_set_fault(qo_sim *s, const double *a, const double *b,
                      const double *eta, const double *Tau_n0,
                      const double *SlipShift, const double *tau0,
                      const double *Slip, const double *psi, double f0,
                      double V0, double L, double Vini) {
    const size_t n = (size_t)s->nz * sizeof(double);
    memcpy(s->a, a, n); memcpy(s->b, b, n); memcpy(s->eta, eta, n);
    memcpy(s->Tau_n0, Tau_n0, n); memcpy(s->SlipShift, SlipShift, n);
    memcpy(s->Slip, Slip, n); memcpy(s->psi, psi, n);
    s->have_tau0 = tau0 != NULL;
    if (tau0) memcpy(s->tau0, tau0, n);
    s->f0 = f0; s->V0 = V0; s->L = L; s->Vini = Vini;
}

void qo_sim_set_params(qo_sim *s, double tmax, double ini_dt, double mindt,
                       double maxdt, double totTol, int maxNumSteps) {
    s->tmax = tmax; s->ini_dt = ini_dt; s->mindt = mindt; s->maxdt = maxdt;
    s->totTol = totTol; s->maxNumSteps = maxNumSteps;
}

void qo_sim_set_surface_prolong(qo_sim *s, int v) { s->mg.surface_prolong = v; }
void qo_sim_set_metric(qo_sim *s, const double *jrow) { qo_mg_set_metric(&s->mg, s->nk, jrow); }
void qo_sim_set_coarse_solve(qo_sim *s, int v) { s->mg.coarse_solve = v; }

void qo_sim_set_U(qo_sim *s, const double *U) {
    memcpy(s->U, U, (size_t)s->nx * s->nz * sizeof(double));
}

/* ode_solve(): multigrid() then extend_crew(), odeSolver.cpp:605-609. */
static int sim_solve(qo_sim *s) {
    qo_pack(s->ni, s->nk, s->U, s->u);
    double rn;
    const int cyc = s->hook ? s->hook(s->hook_ctx, s->u, s->ni, s->nk, &rn)
                            : qo_multigrid(&s->mg, s->u, s->f, s->tol_mode, s->tol, s->max_cycles, &rn, NULL);
    qo_unpack(s->ni, s->nk, s->u, s->U);
    qo_extend_crew(s->ni, s->nk, s->U);
    s->solves++;
    s->vcycles += cyc;
    if (s->max_cycles > 0 && cyc >= s->max_cycles && !(rn <= s->tol) && s->status == 0) s->status = 1;
    return 0;
}

/* One stage tail: stress, NRsearch, cal_dpsi (e.g. odeSolver.cpp:1498-1500). */
static int sim_fault(qo_sim *s, const double *psi, double *V, double *dpsi) {
    qo_eval_stress_on_fault(s->ni, s->nk, s->dh, s->U, s->mu_node, s->Tau_n0, s->Ts, s->Tn);
    const int st = qo_nrsearch(s->nk, s->Ts, s->Tn, s->have_tau0 ? s->tau0 : NULL, s->a, s->eta,
                               psi, s->V0, V, s->iters);
    for (int k = 1; k <= s->nk; k++) s->newton_iters += s->iters[k];
    qo_cal_dpsi(s->nk, psi, s->b, V, s->f0, s->V0, s->L, dpsi);
    if (st != 0 && s->status == 0) s->status = st;
    return st;
}

int qo_sim_solve(qo_sim *s) { return sim_solve(s); }

int qo_sim_start(qo_sim *s) {
    s->dt = s->ini_dt;                                             /* :1363 */
    for (int k = 1; k <= s->nk; k++) {                             /* :1428-1432 */
        s->kslip[1][k] = s->Slip[k];
        s->kpsi[1][k] = s->psi[k];
    }
    qo_set_boundary(s->ni, s->nk, s->U, s->kslip[1], s->SlipShift, s->Vini, s->t, 0.0, s->dt);
    sim_solve(s);
    return sim_fault(s, s->kpsi[1], s->fV[1], s->fdpsi[1]);
}

/* Restart from the fault state an accepted step leaves behind (Slip, psi,
 * t, dt, the error history, the step count): zero Newton seeds as after the
 * commit (odeSolver.cpp:1605-1614), then the commit's refresh solve and
 * fault update (:1615-1619) from the current U as the guess. */
int qo_sim_resume(qo_sim *s, const double *Slip, const double *psi, double t, double dt,
                  double errA0, double errA1, int it) {
    const size_t nzb = (size_t)s->nz * sizeof(double);
    memcpy(s->Slip, Slip, nzb);
    memcpy(s->psi, psi, nzb);
    for (int st = 1; st <= 6; st++) {
        memset(s->kslip[st], 0, nzb); memset(s->kpsi[st], 0, nzb);
        memset(s->fV[st], 0, nzb); memset(s->fdpsi[st], 0, nzb);
    }
    for (int k = 1; k <= s->nk; k++) {
        s->kslip[1][k] = s->Slip[k];
        s->kpsi[1][k] = s->psi[k];
    }
    s->t = t; s->dt = dt; s->errA[0] = errA0; s->errA[1] = errA1; s->it = it;
    s->status = 0;
    qo_set_boundary(s->ni, s->nk, s->U, s->kslip[1], s->SlipShift, s->Vini, s->t, 0.0, s->dt);
    sim_solve(s);
    return sim_fault(s, s->kpsi[1], s->fV[1], s->fdpsi[1]);
}

int qo_sim_step(qo_sim *s) {
    const int nk = s->nk;
    const size_t nzb = (size_t)s->nz * sizeof(double);
    double totErr = 0.0;
    s->it = s->it + 1;                                             /* :1464 */
    int attemptCount = 0;
    while (attemptCount < 100) {                                   /* :1466 */
        attemptCount++;
        s->attempts++;
        if (s->t + s->dt > s->tmax) s->dt = s->tmax - s->t;        /* :1473-1476 */
        for (int st = 2; st <= 6; st++) {                          /* :1477-1488 */
            memset(s->kslip[st], 0, nzb); memset(s->kpsi[st], 0, nzb);
            memset(s->fV[st], 0, nzb); memset(s->fdpsi[st], 0, nzb);
        }
        memset(s->y3s, 0, nzb); memset(s->y3p, 0, nzb);
        memset(s->y4s, 0, nzb); memset(s->y4p, 0, nzb);
        for (int st = 2; st <= 6; st++) {                          /* :1491-1566 */
            double *ks = s->kslip[st], *kp = s->kpsi[st];
            for (int k = 1; k <= nk; k++) {
                ks[k] = s->Slip[k] + RK_A[st][1] * s->dt * s->fV[1][k];
                for (int j = 2; j < st; j++) ks[k] = ks[k] + RK_A[st][j] * s->dt * s->fV[j][k];
                kp[k] = s->psi[k] + RK_A[st][1] * s->dt * s->fdpsi[1][k];
                for (int j = 2; j < st; j++) kp[k] = kp[k] + RK_A[st][j] * s->dt * s->fdpsi[j][k];
            }
            qo_set_boundary(s->ni, nk, s->U, ks, s->SlipShift, s->Vini, s->t, RK_C[st], s->dt);
            sim_solve(s);
            sim_fault(s, kp, s->fV[st], s->fdpsi[st]);
        }
        for (int k = 1; k <= nk; k++) {                            /* :1569-1593 */
            s->y3s[k] = s->Slip[k] + RK_HB[1] * s->dt * s->fV[1][k];
            s->y4s[k] = s->Slip[k] + RK_B[1] * s->dt * s->fV[1][k];
            s->y3p[k] = s->psi[k] + RK_HB[1] * s->dt * s->fdpsi[1][k];
            s->y4p[k] = s->psi[k] + RK_B[1] * s->dt * s->fdpsi[1][k];
            for (int j = 3; j <= 6; j++) {
                s->y3s[k] = s->y3s[k] + RK_HB[j] * s->dt * s->fV[j][k];
                s->y3p[k] = s->y3p[k] + RK_HB[j] * s->dt * s->fdpsi[j][k];
                s->y4s[k] = s->y4s[k] + RK_B[j] * s->dt * s->fV[j][k];
                s->y4p[k] = s->y4p[k] + RK_B[j] * s->dt * s->fdpsi[j][k];
            }
        }
        totErr = qo_compute_error(nk, s->y3s, s->y3p, s->y4s, s->y4p);   /* :1595 */
        if (totErr < s->totTol) break;
        s->dt = step_size_guarded(s->it, s->dt, s->mindt, s->maxdt, totErr, s->totTol, s->errA);
        if (s->mindt == s->dt) break;                              /* :1602 */
    }
    s->t = s->t + s->dt;                                           /* :1605 */
    for (int k = 1; k <= nk; k++) {
        s->Slip[k] = s->y4s[k]; s->kslip[1][k] = s->y4s[k]; s->fV[1][k] = 0.0;
        s->psi[k] = s->y4p[k]; s->kpsi[1][k] = s->y4p[k]; s->fdpsi[1][k] = 0.0;
    }
    qo_set_boundary(s->ni, nk, s->U, s->kslip[1], s->SlipShift, s->Vini, s->t, 0.0, s->dt);
    sim_solve(s);
    sim_fault(s, s->kpsi[1], s->fV[1], s->fdpsi[1]);
    double newDeltaT;
    if (totErr != 0.0)                                             /* :1621-1632 */
        newDeltaT = step_size_guarded(s->it, s->dt, s->mindt, s->maxdt, totErr, s->totTol, s->errA);
    else
        newDeltaT = s->dt;
    s->errA[1] = s->errA[0];
    s->errA[0] = totErr;
    s->dt = newDeltaT;
    return s->status;
}

void qo_sim_get(const qo_sim *s, double *U, double *Slip, double *psi,
                double *V, double *Ts, double *dpsi) {
    const size_t nzb = (size_t)s->nz * sizeof(double);
    if (U) memcpy(U, s->U, (size_t)s->nx * s->nz * sizeof(double));
    if (Slip) memcpy(Slip, s->Slip, nzb);
    if (psi) memcpy(psi, s->psi, nzb);
    if (V) memcpy(V, s->fV[1], nzb);
    if (Ts) memcpy(Ts, s->Ts, nzb);
    if (dpsi) memcpy(dpsi, s->fdpsi[1], nzb);
}

void qo_sim_scalars(const qo_sim *s, double *d, long long *iv) {
    if (d) { d[0] = s->t; d[1] = s->dt; d[2] = s->errA[0]; d[3] = s->errA[1]; }
    if (iv) {
        iv[0] = s->it; iv[1] = s->solves; iv[2] = s->vcycles; iv[3] = s->attempts;
        iv[4] = s->newton_iters; iv[5] = s->status;
    }
}

void qo_sim_set_scalars(qo_sim *s, double t, double dt, double errA0,
                        double errA1, int it) {
    s->t = t; s->dt = dt; s->errA[0] = errA0; s->errA[1] = errA1; s->it = it;
}
