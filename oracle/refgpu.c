/*
 * refgpu.c -- the reference's own GPU multigrid, for timing it as a baseline.
 *
 * TEST / BASELINE INFRASTRUCTURE ONLY.  Only bench.py's --impl reference
 * arm and tests/ load it; the product library never does.
 *
 * The reference's five CUDA kernels (odeSolver.cpp:757-1099) are compiled
 * unmodified by oracle/Makefile into _ref/ref_kernels.cubin.  This file is
 * the host side around them, restating the reference's host functions in C:
 *   - the level tables of RK43's GPU initialisation (odeSolver.cpp:1384-1420)
 *     into the cubin's __constant__ dimsinfo_dev / innersinfo_dev;
 *   - smooth(), vcycle() (:741-755, :1101-1147) with the reference's
 *     hard-coded n_levels = 6, n_cycles = 32 and 32 x 16 blocks;
 *   - multigrid() (:652-720): u host-to-device every solve, the residual
 *     norm by calcuDelta_dev + cublasDnrm2 after every V-cycle (a blocking
 *     read), device-to-host at the end.
 * It plugs into the CPU oracle's RK43 loop as its solve hook
 * (qo_sim_set_solve_hook), which runs the reference's host code for the
 * rest of each stage -- the reference program's own split.
 *
 * The stopping rule is the reference's (||r||2 <= eps), with eps either the
 * reference's absolute 1e-9 or tol * ||r(u_interior = 0)||2 (the relative
 * tolerance of the GPU solvers it is compared with), the zero-interior
 * residual taken from the boundary columns on the host.
 *
 * Built against the CUDA driver API and cuBLAS only (no runtime API):
 *   gcc -O2 -fPIC -shared refgpu.c -lcuda -lcublas
 */
#include <cublas_v2.h>
#include <cuda.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define RG_LEVELS 6   /* odeSolver.cpp:3 */
#define RG_CYCLES 32  /* odeSolver.cpp:4 */

typedef struct { int M, N, K, fin_coa; double DH; } rg_diminfo;           /* struct.h:81-87 */
typedef struct { int istart, iend, jstart, jend, kstart, kend; } rg_inners; /* struct.h:90-97 */

typedef struct refgpu {
    CUcontext ctx;
    CUmodule mod;
    CUfunction rb0, rb1, res, restr, prol, delta;
    cublasHandle_t blas;
    rg_diminfo dims[RG_LEVELS];
    rg_inners inn[RG_LEVELS];
    CUdeviceptr u, f, mu, dres, res_l[RG_LEVELS], res2[RG_LEVELS], err2[RG_LEVELS];
    int ni, nk, nx;
    double dh, tol;
    int rel;
    const double *mu_host;
    double *f_host;        /* the right-hand side the reference copies up every solve (zero) */
    long long solves, vcycles;
    char err[256];
} refgpu;

static int chk(refgpu *g, CUresult r, const char *what) {
    if (r != CUDA_SUCCESS) {
        const char *s = NULL;
        cuGetErrorString(r, &s);
        snprintf(g->err, sizeof(g->err), "%s: %s", what, s ? s : "?");
        return -1;
    }
    return 0;
}

const char *rg_last_error(refgpu *g) { return g ? g->err : "no handle"; }

static int launch(refgpu *g, CUfunction f, unsigned gx, unsigned gy, void **args) {
    return chk(g, cuLaunchKernel(f, gx, gy, 1, 32, 16, 1, 0, NULL, args, NULL), "cuLaunchKernel");
}

static unsigned cdv(int n, int b) { return (unsigned)((n + b - 1) / b); }

static unsigned gx_of(const refgpu *g, int l) { return cdv(g->inn[l].kend - g->inn[l].kstart, 32); }
static unsigned gy_of(const refgpu *g, int l) { return cdv(g->inn[l].jend - g->inn[l].jstart, 16); }

/* smooth(), odeSolver.cpp:741-755 */
static int smooth(refgpu *g, CUdeviceptr u, CUdeviceptr f, int level) {
    void *a[] = {&u, &f, &g->mu, &level};
    for (int it = 0; it < RG_CYCLES; it++) {
        if (launch(g, g->rb0, gx_of(g, level), gy_of(g, level), a)) return -1;
        if (launch(g, g->rb1, gx_of(g, level), gy_of(g, level), a)) return -1;
    }
    return 0;
}

/* vcycle(), odeSolver.cpp:1101-1147 */
static int vcycle(refgpu *g, CUdeviceptr u, CUdeviceptr f, int level) {
    if (level >= RG_LEVELS - 1) return smooth(g, u, f, level);
    CUdeviceptr r = g->res_l[level], r2 = g->res2[level], e2 = g->err2[level];
    if (smooth(g, u, f, level)) return -1;
    void *ar[] = {&r, &u, &f, &g->mu, &level};
    if (launch(g, g->res, gx_of(g, level), gy_of(g, level), ar)) return -1;
    int l1 = level + 1;
    const rg_diminfo *c = &g->dims[l1];
    void *as[] = {&r2, &r, &e2, &l1};
    if (launch(g, g->restr, cdv(c->K - 2, 32), cdv(c->N, 16), as)) return -1;
    if (vcycle(g, e2, r2, l1)) return -1;
    void *ap[] = {&u, &e2, &l1};
    if (launch(g, g->prol, cdv(c->K - 1, 32), cdv(c->N - 1, 16), ap)) return -1;
    return smooth(g, u, f, level);
}

/* calcuDelta_dev + cublasDnrm2 (odeSolver.cpp:693-694) */
static int delta_norm(refgpu *g, double *out) {
    int l0 = 0;
    void *a[] = {&g->u, &g->f, &g->mu, &g->dres, &l0};
    if (launch(g, g->delta, gx_of(g, 0), gy_of(g, 0), a)) return -1;
    if (cublasDnrm2(g->blas, g->nk * g->ni, (const double *)(uintptr_t)g->dres, 1, out) != CUBLAS_STATUS_SUCCESS) {
        snprintf(g->err, sizeof(g->err), "cublasDnrm2 failed");
        return -1;
    }
    return 0;
}

/* ||r(u_interior = 0)||2 of the packed u: only the columns next to the
 * Dirichlet data see a residual, -(mu_face u_boundary) / h^2 (the level-0
 * x-face moduli of calcuDelta_dev, odeSolver.cpp:1061-1063). */
static double r0_norm(const refgpu *g, const double *u) {
    const long W = 2L * g->nx - 1;
    const int K = g->ni;
    const double h2 = g->dh * g->dh;
    double s = 0.0;
    for (int j = 0; j < g->nk; j++) {
        const long row = (long)(j + 1) * 2 * W;
        if (K - 2 == 1) {
            const double r = -(g->mu_host[3 + row] * u[(long)j * K] + g->mu_host[5 + row] * u[(long)j * K + 2]) / h2;
            s += r * r;
        } else {
            const double r1 = -(g->mu_host[3 + row] * u[(long)j * K]) / h2;
            const double r2 = -(g->mu_host[(K - 1) * 2 + 1 + row] * u[(long)j * K + K - 1]) / h2;
            s += r1 * r1 + r2 * r2;
        }
    }
    return sqrt(s);
}

/* multigrid()'s device part, odeSolver.cpp:682-707: the packed u in, solved
 * u out; returns the V-cycles (the oracle's solve-hook signature). */
int rg_solve(void *ctx, double *u, int ni, int nk, double *rnorm) {
    refgpu *g = (refgpu *)ctx;
    if (ni != g->ni || nk != g->nk) return -1;
    const size_t bytes = sizeof(double) * (size_t)ni * nk;
    if (chk(g, cuCtxSetCurrent(g->ctx), "cuCtxSetCurrent")) return -1;
    if (chk(g, cuMemcpyHtoD(g->u, u, bytes), "H2D u")) return -1;
    if (chk(g, cuMemcpyHtoD(g->f, g->f_host, bytes), "H2D f")) return -1;   /* f_host: zero on level 0 */
    const double eps = g->rel ? g->tol * r0_norm(g, u) : g->tol;
    double delta = 1.0;
    int cyc = 0;
    if (delta_norm(g, &delta)) return -1;
    while (delta > eps && cyc < 100000) {
        if (vcycle(g, g->u, g->f, 0)) return -1;
        if (delta_norm(g, &delta)) return -1;
        cyc++;
    }
    if (chk(g, cuMemcpyDtoH(u, g->u, bytes), "D2H u")) return -1;
    if (rnorm) *rnorm = delta;
    g->solves++;
    g->vcycles += cyc;
    return cyc;
}

void rg_stats(const refgpu *g, long long *out2) {
    out2[0] = g->solves;
    out2[1] = g->vcycles;
}

void rg_free(refgpu *g) {
    if (!g) return;
    if (g->ctx) cuCtxSetCurrent(g->ctx);
    CUdeviceptr *bufs[] = {&g->u, &g->f, &g->mu, &g->dres};
    for (int i = 0; i < 4; i++)
        if (*bufs[i]) cuMemFree(*bufs[i]);
    for (int l = 0; l < RG_LEVELS; l++) {
        if (g->res_l[l]) cuMemFree(g->res_l[l]);
        if (g->res2[l]) cuMemFree(g->res2[l]);
        if (g->err2[l]) cuMemFree(g->err2[l]);
    }
    if (g->blas) cublasDestroy(g->blas);
    free(g->f_host);
    if (g->mod) cuModuleUnload(g->mod);
    if (g->ctx) {
        CUdevice dev;
        if (cuCtxGetDevice(&dev) == CUDA_SUCCESS) cuDevicePrimaryCtxRelease(dev);
    }
    free(g);
}

static int alloc0(refgpu *g, CUdeviceptr *p, size_t n) {
    if (chk(g, cuMemAlloc(p, n * sizeof(double)), "cuMemAlloc")) return -1;
    return chk(g, cuMemsetD8(*p, 0, n * sizeof(double)), "cuMemset");
}

/* RK43's GPU initialisation (odeSolver.cpp:1365-1425) for an ni x nk grid
 * of spacing dh and the staggered mu_equi (2nx-1)(2nz-1); rel = 1: stop at
 * tol * ||r0||, rel = 0: at tol (the reference: 1e-9). */
refgpu *rg_create(const char *cubin, int ni, int nk, double dh, const double *mu_equi, int rel, double tol,
                  char *err, int errlen) {
    refgpu *g = (refgpu *)calloc(1, sizeof(refgpu));
    g->f_host = (double *)calloc((size_t)ni * nk, sizeof(double));
    g->ni = ni; g->nk = nk; g->nx = ni + 2; g->dh = dh; g->rel = rel; g->tol = tol; g->mu_host = mu_equi;
    CUdevice dev;
    int ok = !chk(g, cuInit(0), "cuInit") && !chk(g, cuDeviceGet(&dev, 0), "cuDeviceGet") &&
             !chk(g, cuDevicePrimaryCtxRetain(&g->ctx, dev), "cuDevicePrimaryCtxRetain") &&
             !chk(g, cuCtxSetCurrent(g->ctx), "cuCtxSetCurrent") &&
             !chk(g, cuModuleLoad(&g->mod, cubin), "cuModuleLoad");
    static const char *names[6] = {"_Z11rbgs_kernelILi0EEvPdS0_S0_i", "_Z11rbgs_kernelILi1EEvPdS0_S0_i",
                                   "_Z15residual_kernelPdS_S_S_i", "_Z18restriction_kernelPdS_S_i",
                                   "_Z17prolongate_kernelPdS_i", "_Z14calcuDelta_devPdS_S_S_i"};
    CUfunction *fns[6] = {&g->rb0, &g->rb1, &g->res, &g->restr, &g->prol, &g->delta};
    for (int i = 0; ok && i < 6; i++) ok = !chk(g, cuModuleGetFunction(fns[i], g->mod, names[i]), names[i]);
    if (ok) {
        int n = nk, k = ni;
        double h = dh;
        g->dims[0].M = 1; g->dims[0].N = n; g->dims[0].K = k; g->dims[0].fin_coa = 1; g->dims[0].DH = h;
        for (int i = 0; i < RG_LEVELS - 1; i++) {
            n = (n - 1) / 2 + 1; k = (k - 1) / 2 + 1; h *= 2;
            g->dims[i + 1].M = 1; g->dims[i + 1].N = n; g->dims[i + 1].K = k;
            g->dims[i + 1].fin_coa = 1 << (i + 1); g->dims[i + 1].DH = h;
        }
        for (int i = 0; i < RG_LEVELS; i++) {
            g->inn[i].istart = 0; g->inn[i].iend = 1; g->inn[i].jstart = 0; g->inn[i].jend = g->dims[i].N;
            g->inn[i].kstart = 1; g->inn[i].kend = g->dims[i].K - 1;
        }
        CUdeviceptr p;
        size_t sz;
        ok = !chk(g, cuModuleGetGlobal(&p, &sz, g->mod, "dimsinfo_dev"), "dimsinfo_dev") &&
             sz == sizeof(g->dims) && !chk(g, cuMemcpyHtoD(p, g->dims, sizeof(g->dims)), "dims") &&
             !chk(g, cuModuleGetGlobal(&p, &sz, g->mod, "innersinfo_dev"), "innersinfo_dev") &&
             sz == sizeof(g->inn) && !chk(g, cuMemcpyHtoD(p, g->inn, sizeof(g->inn)), "inners");
        if (!ok && !g->err[0]) snprintf(g->err, sizeof(g->err), "constant table size mismatch");
    }
    const size_t nmu = (size_t)(2 * (ni + 2) - 1) * (2 * (nk + 2) - 1);
    if (ok) ok = !alloc0(g, &g->u, (size_t)ni * nk) && !alloc0(g, &g->f, (size_t)ni * nk) &&
                 !alloc0(g, &g->dres, (size_t)ni * nk) && !alloc0(g, &g->mu, nmu) &&
                 !chk(g, cuMemcpyHtoD(g->mu, mu_equi, nmu * sizeof(double)), "H2D mu");
    for (int i = 0; ok && i < RG_LEVELS - 1; i++)
        ok = !alloc0(g, &g->res_l[i], (size_t)g->dims[i].N * g->dims[i].K) &&
             !alloc0(g, &g->res2[i], (size_t)g->dims[i + 1].N * g->dims[i + 1].K) &&
             !alloc0(g, &g->err2[i], (size_t)g->dims[i + 1].N * g->dims[i + 1].K);
    if (ok && cublasCreate(&g->blas) != CUBLAS_STATUS_SUCCESS) {
        snprintf(g->err, sizeof(g->err), "cublasCreate failed");
        ok = 0;
    }
    if (!ok) {
        if (err) snprintf(err, errlen, "%s", g->err);
        rg_free(g);
        return NULL;
    }
    return g;
}
