// fault.cu -- fault-node kernels of the RK43 stage pipeline: stage
// combination + boundary data, shear stress from u, Newton for slip rate,
// aging law, embedded error estimate and step commit.  One thread per fault
// node; nodes are independent (fault.cpp:139-232, odeSolver.cpp:1150-1238).
#include <math.h>

#include "hist_fit.cuh"

namespace qd {

// Explicit ARK4(3)6L tableau of the reference's integrator
// (odeSolver.cpp:1298-1334); published coefficients, kept identical.
void rk_tableau(double c[7], double b[7], double hb[7], double a[7][7]) {
    for (int i = 0; i < 7; i++) {
        c[i] = b[i] = hb[i] = 0.0;
        for (int j = 0; j < 7; j++) a[i][j] = 0.0;
    }
    c[2] = 1. / 2.; c[3] = 83. / 250.; c[4] = 31. / 50.; c[5] = 17. / 20.; c[6] = 1.;
    b[1] = 82889. / 524892.; b[3] = 15625. / 83664.; b[4] = 69875. / 102672.;
    b[5] = -2260. / 8211.; b[6] = 1. / 4.;
    hb[1] = 4586570599. / 29645900160.; hb[3] = 178811875. / 945068544.;
    hb[4] = 814220225. / 1159782912.; hb[5] = -3700637. / 11593932.; hb[6] = 61727. / 225920.;
    a[2][1] = 1. / 2.;
    a[3][1] = 13861. / 62500.; a[3][2] = 6889. / 62500.;
    a[4][1] = -116923316275. / 2393684061468.; a[4][2] = -2731218467317. / 15368042101831.;
    a[4][3] = 9408046702089. / 11113171139209.;
    a[5][1] = -451086348788. / 2902428689909.; a[5][2] = -2682348792572. / 7519795681897.;
    a[5][3] = 12662868775082. / 11960479115383.; a[5][4] = 3355817975965. / 11060851509271.;
    a[6][1] = 647845179188. / 3216320057751.; a[6][2] = 73281519250. / 8382639484533.;
    a[6][3] = 552539513391. / 3454668386233.; a[6][4] = 3354512671639. / 8306763924573.;
    a[6][5] = 4040. / 17871.;
}

struct RkCoefs {
    double c[7], b[7], hb[7], a[7][7];
};
__constant__ RkCoefs c_rk;
static bool g_rk_uploaded = false;

static int upload_tableau(qd_solver *s) {
    if (g_rk_uploaded) return QD_OK;
    RkCoefs h;
    rk_tableau(h.c, h.b, h.hb, h.a);
    QD_CUDA(cudaMemcpyToSymbol(c_rk, &h, sizeof(h)));
    g_rk_uploaded = true;
    (void)s;
    return QD_OK;
}

struct FaultArgs {
    int nk, K, P;
    double dh;
    double *u0;  // level-0 displacement (compact, pitched)
    FaultState F;
    DevStatus *status;
    int start32;    // Newton start: 0 the reference's x = 0, 1 newton_start32
};

static FaultArgs fargs(qd_solver *s) {
    FaultArgs a;
    a.nk = s->nk; a.K = s->dims[0].K; a.P = s->dims[0].P; a.dh = s->dh;
    a.u0 = s->L64[0].u; a.F = s->F; a.status = s->d_status;
    a.start32 = s->newton_start;
    return a;
}

static inline int nblk(int n, int b) { return (n + b - 1) / b; }

// ---------------------------------------------------------------------------
// device physics
// ---------------------------------------------------------------------------

// partial1st + eval_stress_on_fault (fault.cpp:153,162): one-sided SBP-4
// closure derivative at the fault column, GPa * (m/m) * 1e3 -> MPa.
__device__ __forceinline__ double fault_stress(const double *urow, double mu, double dh) {
    const double du = (-24.0 / (17.0 * dh)) * urow[0] + (59.0 / (34.0 * dh)) * urow[1] +
                      (-4.0 / (17.0 * dh)) * urow[2] + (-3.0 / (34.0 * dh)) * urow[3];
    return mu * du * 1.0e3;
}

// log(sinh(y)) for y > 0 without overflow
__device__ __forceinline__ double log_sinh(double y) {
    return y > 20.0 ? y - 0.69314718055994531 + log1p(-exp(-2.0 * y)) : log(sinh(y));
}

// A single-precision start for the Newton iteration below (the solver's
// Newton start mode 1).  With y = |x|, Y = |fb|/fa and r = Y - y the
// equation is  (A/fa) sinh y = r  on 0 < y < Y, carried through ln(A/fa)
// (A = 2 eta V0 e^{-psi/a} leaves binary32's range).  Each step is Newton on
// the form that is nearly linear where the step is taken: the equation as
// it stands, (A/fa) sinh y - r, where (A/fa) cosh y < 1 (the linear term
// dominates its slope), and its log form  ln(A/fa) + ln sinh y - ln r
// elsewhere (the exponential dominates: there the reference's iteration
// from x = 0 walks down the exponential one unit of x per step, up to 11
// steps near a rupture front).  Both are increasing in y; a step that
// leaves the shrinking sign bracket bisects it.  The start is the least of
// Y and ln(2|fb|/A + 1), both upper bounds of the root (sinh y >= (e^y -
// 1)/2); at most 12 steps, to a relative step of 1e-6.  In binary32 on the
// FP32 pipe this costs little against one FP64 step (GB300's FP64 pipe
// issues about one instruction per SM clock).  The inputs are rounded on
// the integer pipes (d2f_rne).  Returns x = sign(fb) y, or 0 (the
// reference's seed) when fb = 0 or nothing finite came out.
__device__ double newton_start32(double Ts, double Tn, double tau0, double a, double eta, double psi,
                                 double V0) {
    const float fb = d2f_rne(Ts + tau0), af = d2f_rne(a);
    const float fa = af * fabsf(d2f_rne(Tn)), afb = fabsf(fb);
    const float lnA = logf(2.f * d2f_rne(eta) * d2f_rne(V0)) - d2f_rne(psi) / af;
    const float lnAf = lnA - logf(fa);                          // ln(A / fa)
    const float Y = afb / fa;
    if (!(Y > 0.f) || !isfinite(Y) || !isfinite(lnAf)) return 0.0;
    const float t = 0.6931472f + logf(afb) - lnA;              // ln(2|fb|/A)
    float y = fminf(Y, t > 15.f ? t : log1pf(expf(t)));
    float ylo = 0.f, yhi = Y;
    for (int it = 0; it < 12; it++) {
        float ls, lc;                                           // ln sinh y, ln cosh y
        if (y > 15.f) {
            ls = lc = y - 0.6931472f;
        } else {
            ls = logf(sinhf(y));
            lc = logf(coshf(y));
        }
        const float q = expf(fminf(lnAf + lc, 80.f));          // (A/fa) cosh y
        const float r = Y - y;
        float yn;
        if (q < 1.f || !(r > 0.f)) {
            const float g = expf(fminf(lnAf + ls, 80.f)) - r;
            if (g > 0.f) yhi = fminf(yhi, y); else ylo = fmaxf(ylo, y);
            yn = y - g / (q + 1.f);
        } else {
            const float G = lnAf + ls - logf(r);
            if (G > 0.f) yhi = fminf(yhi, y); else ylo = fmaxf(ylo, y);
            yn = y - G / (1.f / tanhf(y) + 1.f / r);
        }
        if (!(yn >= ylo && yn <= yhi)) yn = 0.5f * (ylo + yhi);
        const bool done = fabsf(yn - y) <= 1e-6f * y;
        y = yn;
        if (done) break;
    }
    if (!(y > 0.f) || !isfinite(y)) return 0.0;
    const double x = f2d_exact(y);
    return fb > 0.f ? x : -x;
}

// NRsearch (fault.cpp:180-228) for one node, safeguarded.  Unknown
// x = asinh(V e^{psi/a} / 2V0); residual g(x) = A sinh x + fa x - fb with
// A = 2 eta V0 e^{-psi/a} > 0, fa = a |sigma_n| > 0, so g is increasing and
// the root lies in the bracket between 0 and fb/fa.
// Phase 1 is the reference's Newton step and stopping rule; from the
// reference's seed (x = 0) its iterates never leave the bracket (by more
// than a few ulps, where an end of the bracket is the root), so they are
// the reference's.  If a step leaves the bracket or overflows (the reference
// then produces NaN and exits), phase 2 takes over: Newton on
// G(y) = ln(A sinh y) - ln(|fb| - fa y), y = |x|, which is nearly linear
// where sinh is exponential, with bisection whenever a step leaves the
// shrinking bracket.  start32: with the reference's zero seed, start from
// newton_start32 instead (clamped into the bracket); the iteration and its
// stopping rule are the same, so it ends at the same root in fewer FP64
// steps (iters counts the FP64 steps).  Each dependent FP64 instruction
// waits about 130 clocks for the one before it on GB300, so this path also
// shortens the chain: e^{|x| - pa} is carried from step to step by the
// step's small factor (exp_small) instead of a new exponential, the
// division of the step is div_refined, and the aging law's exponential
// (*ag = e^{ag_arg}, when ag is not null) is taken beside the first
// exponential, where the two chains overlap.
__device__ __forceinline__ double newton_v(double Ts, double Tn, double tau0, double a, double eta, double psi,
                           double V0, double Vseed, int *iters, unsigned int *flags, bool start32 = false,
                           double ag_arg = 0.0, double *ag = nullptr) {
    const double pa = psi / a;
    const double fa = a * fabs(Tn);
    const double fb = Ts + tau0;
    // A = 2 eta V0 e^{-pa}, formed where it is used: with the binary32
    // start, |x| > 20 (nearly every node) needs only eta V0 e^{|x| - pa}
    double A = -1.0;
    auto coefA = [&]() {
        if (A < 0.0) A = 2.0 * eta * V0 * exp(-pa);
        return A;
    };
    double lo, hi;
    if (fb >= 0.0) { lo = 0.0; hi = fb / fa; } else { lo = fb / fa; hi = 0.0; }
    // the seed's x; a zero seed (the reference's, every stage after the
    // first) gives x = +0 without the exponential and asinh while e^{psi/a}
    // is finite, the same value the full expression gives
    double x;
    if (start32 && Vseed == 0.0)
        x = fmin(fmax(newton_start32(Ts, Tn, tau0, a, eta, psi, V0), lo), hi);
    else
        x = (Vseed == 0.0 && pa < 709.0) ? 0.0 : asinh(0.5 * Vseed / V0 * exp(pa));
    if (!(x >= lo && x <= hi)) x = 0.5 * (lo + hi);
    // e^{|x| - pa} for the current x while |x| > 20 (binary32 start), else < 0
    double E = -1.0;
    if (start32 && fabs(x) > 20.0) {
        E = exp(fabs(x) - pa);
        if (ag) *ag = exp(ag_arg);
        ag = nullptr;
    }
    const int itmax = 200;
    int it = 0;
    bool done = false, phase2 = false;
    while (it < itmax) {
        double as, ac;   // A sinh x, A cosh x
        if (start32 && fabs(x) > 20.0) {
            // e^{-2|x|} < 2^-57: sinh |x| = cosh |x| = e^{|x|}/2 to within
            // the rounding, one exponential instead of three
            if (E < 0.0) E = exp(fabs(x) - pa);
            ac = eta * V0 * E;
            as = x > 0.0 ? ac : -ac;
        } else {
            // sinh(0) = 0 and cosh(0) = 1 exactly: the first step from the
            // reference's zero seed needs neither function
            const bool x0 = x == 0.0;
            as = coefA() * (x0 ? 0.0 : sinh(x));
            ac = coefA() * (x0 ? 1.0 : cosh(x));
        }
        const double fy = as + fa * x - fb;
        const double df = ac + fa;
        const double d = start32 ? -div_refined(fy, df + 1e-100) : -fy / (df + 1e-100);
        const double xn = x + d;
        if (!isnan(fy)) {
            if (fy > 0.0) hi = fmin(hi, x); else lo = fmax(lo, x);
        }
        // a step may end a few ulps past a bracket end that sits on the
        // root (the linear term dominating, or the bracket closed to an
        // ulp): that is where the reference's step ends too, not a step
        // out of the bracket
        const double slack = 4.0 * 2.220446049250313e-16 * fmax(fabs(lo), fabs(hi));
        if (!(xn >= lo - slack && xn <= hi + slack) || isinf(fy) || isnan(fy)) {
            phase2 = true;
            *flags |= ST_NEWTON_BRACKET;
            break;
        }
        // the reference's test |d| / |x| < 1e-10; with the binary32 start
        // the same test without the division
        const bool conv = start32 ? fabs(d) < 1e-10 * (fabs(x) + 1e-100) : fabs(d) / (fabs(x) + 1e-100) < 1e-10;
        it++;
        if (E >= 0.0) {
            const double dd = fabs(xn) - fabs(x);
            E = (fabs(xn) > 20.0 && fabs(dd) <= 1e-3) ? E * exp_small(dd) : -1.0;
        }
        x = xn;
        if (conv) { done = true; break; }
    }
    if (phase2) {
        const double sg = fb >= 0.0 ? 1.0 : -1.0, afb = fabs(fb);
        double ylo = sg > 0.0 ? lo : -hi, yhi = sg > 0.0 ? hi : -lo;
        double y = fmin(fmax(sg * x, ylo), yhi);
        const double lnA = log(coefA());
        while (it < itmax) {
            double yn;
            const double rem = afb - fa * y;
            if (y > 0.0 && rem > 0.0) {
                const double G = lnA + log_sinh(y) - log(rem);
                const double dG = 1.0 / tanh(y) + fa / rem;
                if (G > 0.0) yhi = fmin(yhi, y); else ylo = fmax(ylo, y);
                yn = y - G / dG;
            } else {
                yn = -1.0;   // outside the domain: bisect
            }
            if (!(yn >= ylo && yn <= yhi)) yn = 0.5 * (ylo + yhi);
            const double err = fabs(yn - y) / (fabs(y) + 1e-100);
            it++;
            y = yn;
            if (err < 1e-10) { done = true; break; }
        }
        x = sg * y;
        E = -1.0;
    }
    if (!done) *flags |= ST_NEWTON_CAP;
    *iters = it;
    if (ag) *ag = exp(ag_arg);
    double V;
    if (start32 && fabs(x) > 20.0) {
        V = V0 * (E >= 0.0 ? E : exp(fabs(x) - pa));
        if (x < 0.0) V = -V;
    } else {
        V = 2.0 * V0 * exp(-psi / a);
        V = V * sinh(x);
    }
    if (isnan(V)) *flags |= ST_NEWTON_NAN;
    return V;
}

// cal_dpsi (odeSolver.cpp:1196-1204); aging_from takes its exponential
// A = e^{(f0 - psi)/b} already formed
__device__ __forceinline__ double aging_from(double A, double b, double V, double V0, double L) {
    double d = 0.0;
    if (!isinf(A) && b > 1e-3) d = (b * V0 / L) * (A - V / V0);
    return d;
}

__device__ __forceinline__ double aging(double psi, double b, double V, double f0, double V0,
                                        double L) {
    return aging_from(exp((f0 - psi) / b), b, V, V0, L);
}

__device__ __forceinline__ void report(DevStatus *st, unsigned int flags, int node) {
    if (flags & (ST_NEWTON_NAN | ST_NEWTON_CAP)) {
        atomicOr(&st->flags, flags);
        atomicCAS(&st->bad_node, -1, node);
    } else if (flags) {
        atomicOr(&st->flags, flags);
    }
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// one fault node of k_stage_boundary: the stage's k_s, its Newton seed and
// the two Dirichlet values of row k-1 (also returned in g0, g1)
__device__ __forceinline__ void stage_boundary_node(const FaultArgs &A, int stage, double t, double dt,
                                                    double ratio, int k, double *g0, double *g1) {
    const FaultState &F = A.F;
    double ks = F.Slip[k], kp = F.psi[k];
    if (stage > 1) {
        ks = ks + c_rk.a[stage][1] * dt * F.fV[1][k];
        kp = kp + c_rk.a[stage][1] * dt * F.fdpsi[1][k];
        for (int j = 2; j < stage; j++) {
            ks = ks + c_rk.a[stage][j] * dt * F.fV[j][k];
            kp = kp + c_rk.a[stage][j] * dt * F.fdpsi[j][k];
        }
        F.fV[stage][k] = 0.0;
        F.fdpsi[stage][k] = 0.0;
    }
    F.kslip[stage][k] = ks;
    F.kpsi[stage][k] = kp;
    double *row = A.u0 + (long)(k - 1) * A.P;
    *g0 = 0.5 * ks;
    *g1 = 0.50 * F.Vini * (t + ratio * dt) + F.SlipShift[k];
    row[0] = *g0;
    row[A.K - 1] = *g1;
}

// Stage combination k_s = y + dt sum_j a_sj f_j (odeSolver.cpp:1491-1561),
// the Newton seed of the stage (f_s.V_f, zeroed by the reference, :1484-1488,
// :1610) and setBoundary's two Dirichlet columns (:1162-1172).
// stage 1 copies y (the start and the post-accept refresh, :1430,1606-1614).
// With ND > 0 the same launch also fits the new boundary data by the
// solution history's (hist_fit.cuh): each thread adds its node's two
// boundary values to the normal equations and the last block solves them,
// so the guess needs no launch of its own for the fit.  commit: first the
// accepted step's commit of each node (y <- y4, f_1 zeroed; odeSolver.cpp:
// 1606-1614), which the refresh stage 1 then copies; zero, when not null, is
// set to 0 by one thread (the solve state's need_max at an attempt's first
// stage).
template <int ND>
__global__ void __launch_bounds__(FIT_THREADS)
    k_stage_boundary(FaultArgs A, int stage, double t, double dt, double ratio, FitArgs fit, int commit,
                     double *zero) {
    pdl_trigger();
    pdl_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (zero && blockIdx.x == 0 && threadIdx.x == 0) *zero = 0.0;
    if (commit && k <= A.nk) {
        const FaultState &F = A.F;
        F.Slip[k] = F.y4s[k];
        F.psi[k] = F.y4p[k];
        F.fV[1][k] = 0.0;
        F.fdpsi[1][k] = 0.0;
    }
    if constexpr (ND > 0) {
        FitAcc<ND> acc;
        acc.zero();
        if (k <= A.nk) {
            double g0, g1;
            stage_boundary_node(A, stage, t, dt, ratio, k, &g0, &g1);
            acc.add(fit, k - 1, g0);
            acc.add(fit, fit.N + k - 1, g1);
        }
        fit_reduce_solve<ND>(fit, acc);
    } else if (k <= A.nk) {
        double g0, g1;
        stage_boundary_node(A, stage, t, dt, ratio, k, &g0, &g1);
    }
}

// Blocks past the fault nodes' copy the solved u into a history slot as
// double-float pairs (d_split), and its boundary columns in FP64: the Newton
// chains leave the SMs nearly idle, so the copy rides along instead of
// taking a launch of its own.  Rows are dealt round-robin to the copy
// blocks, 16-byte pairs of nodes across the block's threads, four pairs in
// flight per thread.  The pitch P is even, so every pair is 16-byte aligned
// in both fields.
__device__ __forceinline__ void copy_rows(const CopyJob &J, int blk, int nblk) {
    constexpr int U = 4;
    const int step = 2 * (int)blockDim.x;
    for (int row = blk; row < J.N; row += nblk) {
        const size_t r0 = (size_t)row * J.P;
        for (int c0 = 2 * (int)threadIdx.x; c0 < J.P; c0 += U * step) {
            double2 v[U];
#pragma unroll
            for (int i = 0; i < U; i++) {
                const int c = c0 + i * step;
                if (c < J.P) v[i] = *reinterpret_cast<const double2 *>(J.src + r0 + c);
            }
#pragma unroll
            for (int i = 0; i < U; i++) {
                const int c = c0 + i * step;
                if (c >= J.P) break;
                const float2 a = d_split(v[i].x), b = d_split(v[i].y);
                *reinterpret_cast<float4 *>(J.dst + r0 + c) = make_float4(a.x, a.y, b.x, b.y);
                if (c == 0) J.bc[row] = v[i].x;
                if (c == J.K - 1) J.bc[J.N + row] = v[i].x;
                if (c + 1 == J.K - 1) J.bc[J.N + row] = v[i].y;
            }
        }
    }
}

// stress -> Newton -> aging law for one stage (odeSolver.cpp:1498-1500);
// blocks fault_blocks.. store u into the solution history (job)
__global__ void k_fault_stage(FaultArgs A, int stage, CopyJob job, int fault_blocks) {
    pdl_trigger();
    pdl_wait();
    if ((int)blockIdx.x >= fault_blocks) {
        copy_rows(job, (int)blockIdx.x - fault_blocks, (int)gridDim.x - fault_blocks);
        return;
    }
    const int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (k > A.nk) return;
    const FaultState &F = A.F;
    const double Ts = fault_stress(A.u0 + (long)(k - 1) * A.P, F.mu0[k], A.dh);
    const double Tn = F.Tn0[k];
    F.Ts[k] = Ts;
    F.Tn[k] = Tn;
    const double psi = F.kpsi[stage][k];
    const double bk = F.b[k];
    unsigned int flags = 0;
    int it = 0;
    double agA = 0.0;   // the aging law's exponential, formed inside the Newton solve
    const double V = newton_v(Ts, Tn, F.have_tau0 ? F.tau0[k] : 0.0, F.a[k], F.eta[k], psi, F.V0,
                              F.fV[stage][k], &it, &flags, A.start32 != 0, (F.f0 - psi) / bk, &agA);
    F.fV[stage][k] = V;
    F.fdpsi[stage][k] = aging_from(agA, bk, V, F.V0, F.L);
    F.iters[k] += it;
    report(A.status, flags, k);
}

__global__ void k_stress(FaultArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (k > A.nk) return;
    A.F.Ts[k] = fault_stress(A.u0 + (long)(k - 1) * A.P, A.F.mu0[k], A.dh);
    A.F.Tn[k] = A.F.Tn0[k];
}

__global__ void k_newton(FaultArgs A, const double *Ts, const double *psi, double *V, int *iters) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (k > A.nk) return;
    const FaultState &F = A.F;
    unsigned int flags = 0;
    int it = 0;
    V[k] = newton_v(Ts[k], F.Tn0[k], F.have_tau0 ? F.tau0[k] : 0.0, F.a[k], F.eta[k], psi[k], F.V0,
                    V[k], &it, &flags, A.start32 != 0);
    iters[k] = it;
    report(A.status, flags, k);
}

__global__ void k_dpsi(FaultArgs A, const double *psi, const double *V, double *dpsi) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (k > A.nk) return;
    dpsi[k] = aging(psi[k], A.F.b[k], V[k], A.F.f0, A.F.V0, A.F.L);
}

// y3 / y4 (odeSolver.cpp:1569-1593) and computeError (:1211-1238).  One
// fault node per thread in 32-thread blocks: the nodes' FP64 work spread
// over nk/32 SMs (GB300's FP64 pipe takes about 20 clocks a warp
// instruction per SM); each block's sums into partial[2 block ..], the last
// block to finish adds them in a fixed order (deterministic) and re-arms
// the counter.  inv_sqrt_n = 1/sqrt(nk).  With rep.err set, the last block
// also writes the attempt's report into pinned host memory (the device
// addresses of the solver's host copies): the error, the solve state and
// the status the host reads after its one wait of the attempt.
struct AttemptReport {
    double *err;                 // null: no report
    SolveState *st;
    DevStatus *status;
    const SolveState *d_st;
    const DevStatus *d_status;
};

__global__ void k_error(FaultArgs A, double dt, double *partial, unsigned *count, double inv_sqrt_n, double *out,
                        AttemptReport rep) {
    pdl_wait();
    const FaultState &F = A.F;
    double e1 = 0.0, e2 = 0.0;
    if (const int k = blockIdx.x * blockDim.x + threadIdx.x + 1; k <= A.nk) {
        double y3s = F.Slip[k] + c_rk.hb[1] * dt * F.fV[1][k];
        double y4s = F.Slip[k] + c_rk.b[1] * dt * F.fV[1][k];
        double y3p = F.psi[k] + c_rk.hb[1] * dt * F.fdpsi[1][k];
        double y4p = F.psi[k] + c_rk.b[1] * dt * F.fdpsi[1][k];
        for (int j = 3; j <= 6; j++) {
            y3s = y3s + c_rk.hb[j] * dt * F.fV[j][k];
            y3p = y3p + c_rk.hb[j] * dt * F.fdpsi[j][k];
            y4s = y4s + c_rk.b[j] * dt * F.fV[j][k];
            y4p = y4p + c_rk.b[j] * dt * F.fdpsi[j][k];
        }
        F.y3s[k] = y3s; F.y3p[k] = y3p; F.y4s[k] = y4s; F.y4p[k] = y4p;
        const double t1 = y3s - y4s, t2 = y3p - y4p;
        e1 = t1 * t1;
        e2 = t2 * t2;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e1 += __shfl_down_sync(0xffffffffu, e1, o);
        e2 += __shfl_down_sync(0xffffffffu, e2, o);
    }
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = e1;
        partial[2 * blockIdx.x + 1] = e2;
        __threadfence();
        last = atomicAdd(count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s1 = 0.0, s2 = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += 32) {
        s1 += __ldcg(partial + 2 * b);
        s2 += __ldcg(partial + 2 * b + 1);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_down_sync(0xffffffffu, s1, o);
        s2 += __shfl_down_sync(0xffffffffu, s2, o);
    }
    if (threadIdx.x == 0) {
        *count = 0;
        const double e = sqrt_refined(s1) * inv_sqrt_n + sqrt_refined(s2) * inv_sqrt_n;
        *out = e;
        if (rep.err) {
            *rep.err = e;
            *rep.st = *rep.d_st;
            *rep.status = *rep.d_status;
            __threadfence_system();
        }
    }
}

// ---------------------------------------------------------------------------
// host wrappers
// ---------------------------------------------------------------------------
int fault_alloc(qd_solver *s) {
    const size_t nz = s->nz;
    FaultState &F = s->F;
    double **vecs[] = {&F.mu0, &F.a, &F.b, &F.eta, &F.Tn0, &F.tau0, &F.SlipShift, &F.Slip, &F.psi,
                       &F.Ts, &F.Tn, &F.y3s, &F.y3p, &F.y4s, &F.y4p};
    for (double **p : vecs) {
        if (cudaMalloc(p, nz * sizeof(double)) != cudaSuccess) return QD_ERR_NOMEM;
        QD_CUDA(cudaMemset(*p, 0, nz * sizeof(double)));
    }
    for (int st = 1; st <= 6; st++) {
        double **pp[] = {&F.kslip[st], &F.kpsi[st], &F.fV[st], &F.fdpsi[st]};
        for (double **p : pp) {
            if (cudaMalloc(p, nz * sizeof(double)) != cudaSuccess) return QD_ERR_NOMEM;
            QD_CUDA(cudaMemset(*p, 0, nz * sizeof(double)));
        }
    }
    if (cudaMalloc(&F.iters, nz * sizeof(int)) != cudaSuccess) return QD_ERR_NOMEM;
    QD_CUDA(cudaMemset(F.iters, 0, nz * sizeof(int)));
    return upload_tableau(s);
}

void fault_free(qd_solver *s) {
    FaultState &F = s->F;
    double *vecs[] = {F.mu0, F.a, F.b, F.eta, F.Tn0, F.tau0, F.SlipShift, F.Slip, F.psi,
                      F.Ts, F.Tn, F.y3s, F.y3p, F.y4s, F.y4p};
    for (double *p : vecs) cudaFree(p);
    for (int st = 1; st <= 6; st++) {
        cudaFree(F.kslip[st]); cudaFree(F.kpsi[st]); cudaFree(F.fV[st]); cudaFree(F.fdpsi[st]);
    }
    cudaFree(F.iters);
    s->F = FaultState();
}

// The stage chain's kernels (boundary, history fit and guess, fault stage,
// error estimate) are launched with programmatic stream serialization: each
// waits for its predecessor (pdl_wait) before touching its data, and the
// launch latency between them overlaps the predecessor's tail.
int launch_stage_boundary(qd_solver *s, int stage, double ratio, bool fit, bool commit) {
    FitArgs fa{};
    const int nd = fit ? history_fit_args(s, &fa) : 0;
    // an RK attempt's first stage: the attempt's need_max starts from 0
    double *zero = (stage == 2 && fit) ? &s->d_solve->need_max : nullptr;
    const dim3 grid(nblk(s->nk, FIT_THREADS)), block(FIT_THREADS);
    switch (nd) {
#define QD_SB_CASE(n)                                                                                    \
    case n:                                                                                              \
        QD_CUDA(launch_pdl(true, k_stage_boundary<n>, grid, block, 0, s->stream, fargs(s), stage, s->t, s->dt, \
                           ratio, fa, commit ? 1 : 0, zero));                                            \
        break;
        QD_SB_CASE(0) QD_SB_CASE(1) QD_SB_CASE(2) QD_SB_CASE(3) QD_SB_CASE(4) QD_SB_CASE(5) QD_SB_CASE(6)
        QD_SB_CASE(7)
#undef QD_SB_CASE
        default:
            set_error("stage boundary: %d fit unknowns", nd);
            return QD_ERR_STATE;
    }
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

// The stress/Newton/aging kernels are FP64-pipe bound with one thread per
// fault node: 32-thread blocks spread the nk nodes over nk/32 SMs instead of
// packing four warps onto each of nk/128 SMs' FP64 pipes.
static constexpr int kNewtonBlock = 32;

// copy blocks of the fault-stage launch: eight 32-thread blocks per SM
static constexpr int kCopyBlocks = 1216;

int launch_fault(qd_solver *s, int stage, const CopyJob &job) {
    const int fb = nblk(s->nk, kNewtonBlock);
    const int cb = job.src ? kCopyBlocks : 0;
    QD_CUDA(launch_pdl(true, k_fault_stage, dim3(fb + cb), dim3(kNewtonBlock), 0, s->stream, fargs(s), stage, job,
                       fb));
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

int launch_error(qd_solver *s, bool report) {
    const int nb = nblk(s->nk, 32);
    if (2 * nb > s->n_partial) {
        set_error("error estimate: %d blocks exceed the partial buffer", nb);
        return QD_ERR_ARG;
    }
    AttemptReport rep{};
    if (report) {
        if (!s->dh_scal || !s->dh_solve || !s->dh_status) {
            set_error("error estimate: the pinned host copies are not addressable by the device");
            return QD_ERR_STATE;
        }
        rep.err = s->dh_scal + 2;
        rep.st = s->dh_solve;
        rep.status = s->dh_status;
        rep.d_st = s->d_solve;
        rep.d_status = s->d_status;
    }
    QD_CUDA(launch_pdl(true, k_error, dim3(nb), dim3(32), 0, s->stream, fargs(s), s->dt, s->d_partial, s->d_count,
                       1.0 / sqrt((double)s->nk), s->d_scal + 2, rep));
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}


int launch_stress(qd_solver *s) {
    k_stress<<<nblk(s->nk, 128), 128, 0, s->stream>>>(fargs(s));
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

int launch_newton(qd_solver *s, const double *Ts, const double *psi, double *V, int *iters) {
    k_newton<<<nblk(s->nk, kNewtonBlock), kNewtonBlock, 0, s->stream>>>(fargs(s), Ts, psi, V, iters);
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

int launch_dpsi(qd_solver *s, const double *psi, const double *V, double *dpsi) {
    k_dpsi<<<nblk(s->nk, 128), 128, 0, s->stream>>>(fargs(s), psi, V, dpsi);
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

}  // namespace qd
