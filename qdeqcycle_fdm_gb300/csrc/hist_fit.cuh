// hist_fit.cuh -- the solution-history guess's least-squares fit of new
// boundary data by stored ones (history.cu), shared by the stand-alone fit
// kernel and the stage-boundary kernel that fuses it (fault.cu).
#pragma once

#include "qdeq_internal.cuh"

namespace qd {

static constexpr int HIST_MAX = 8;              // stored solutions
static constexpr int HIST_ND = HIST_MAX - 1;     // fit unknowns at most
static constexpr int FIT_THREADS = 128;          // threads of every block that takes part in a fit
static constexpr int FIT_CTAS = 16;              // blocks of the stand-alone fit kernel
static constexpr int FIT_NA_MAX = HIST_ND * (HIST_ND + 1) / 2 + HIST_ND + 1;

// anchor = slot a, the other stored solutions = slots oth[0..nd)
struct FitArgs {
    const double *u;      // the solver's u with the new boundary data in columns 0, K-1
    const double *bc;     // ring of boundary values
    int N, K, P, a;
    int oth[HIST_ND];
    double *coef, *partial;
    float2 *w;
    unsigned *count;
};

// history.cu: the stage's fit for the boundary kernel (0: no fit)
int history_fit_args(qd_solver *s, FitArgs *F);

// Accumulators of the normal equations over boundary values i (0..2N-1):
// G = D^T D (upper triangle), b = D^T t, |t|^2, with t = g - g_A the new
// data's change from the anchor's and D's column k the k-th stored
// solution's change.
template <int ND>
struct FitAcc {
    static constexpr int NT = ND * (ND + 1) / 2, NA = NT + ND + 1;
    double a[NA];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < NA; i++) a[i] = 0.0;
    }
    __device__ __forceinline__ void add(const FitArgs &F, int i, double g) {
        const int n2 = 2 * F.N;
        const double ga = F.bc[(size_t)F.a * n2 + i], t = g - ga;
        double d[ND];
#pragma unroll
        for (int k = 0; k < ND; k++) d[k] = F.bc[(size_t)F.oth[k] * n2 + i] - ga;
        int q = 0;
#pragma unroll
        for (int k = 0; k < ND; k++)
#pragma unroll
            for (int l = k; l < ND; l++) a[q++] += d[k] * d[l];
#pragma unroll
        for (int k = 0; k < ND; k++) a[NT + k] += d[k] * t;
        a[NA - 1] += t * t;
    }
};

// The fit's reduction and solve, called by every thread of every block of
// a grid of FIT_THREADS-thread blocks after it accumulated its boundary
// values: warp and block sums, then (with more than one block) the last
// block to finish sums the block partials in a fixed order (deterministic),
// and its first thread scales the normal equations to a unit diagonal,
// adds a 1e-12 ridge, solves by Cholesky, keeps the fit only if its misfit
// is below the unfitted change, and writes the coefficients (coef), the
// misfit ratio (coef[HIST_ND]) and the guess's weights as double-float
// pairs (w: the anchor's 1 - sum c, then c).
template <int ND>
__device__ void fit_reduce_solve(const FitArgs &F, FitAcc<ND> &acc) {
    constexpr int NT = FitAcc<ND>::NT, NA = FitAcc<ND>::NA;
    __shared__ double red[FIT_THREADS / 32][NA];
    __shared__ double sums[NA];
    __shared__ int is_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NA; i++) {
        double x = acc.a[i];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][i] = x;
    }
    __syncthreads();
    if (gridDim.x == 1) {
        if (threadIdx.x < NA) {
            double x = 0.0;
            for (int w = 0; w < FIT_THREADS / 32; w++) x += red[w][threadIdx.x];
            sums[threadIdx.x] = x;
        }
        __syncthreads();
        if (threadIdx.x != 0) return;
    } else {
        if (threadIdx.x < NA) {
            double x = 0.0;
            for (int w = 0; w < FIT_THREADS / 32; w++) x += red[w][threadIdx.x];
            F.partial[blockIdx.x * NA + threadIdx.x] = x;
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) is_last = atomicAdd(F.count, 1u) == gridDim.x - 1;
        __syncthreads();
        if (!is_last) return;
        __threadfence();
        if (threadIdx.x < NA) {
            double x = 0.0;
            for (int b = 0; b < (int)gridDim.x; b++) x += __ldcg(F.partial + b * NA + threadIdx.x);
            sums[threadIdx.x] = x;
        }
        __syncthreads();
        if (threadIdx.x != 0) return;
        *F.count = 0;                               // ready for the next fit
    }

    // unit-diagonal scaling, 1e-12 ridge, Cholesky.  This is one thread's
    // chain of FP64 instructions, each waiting about 130 clocks for the one
    // before it on GB300's FP64 pipe, so it avoids FP64 divisions and square
    // roots: the scales are binary32 reciprocal square roots (any scale
    // serves; these make the diagonal 1 to within 1e-7), and each pivot's
    // reciprocal square root r (binary32, refined by one FP64 Newton step)
    // gives both L_jj = p r and the divisions by L_jj as products.
    double G[ND][ND], b[ND], sc[ND], L[ND][ND], rinv[ND], y[ND], c[ND];
    int q = 0;
    for (int k = 0; k < ND; k++)
        for (int l = k; l < ND; l++) {
            G[k][l] = G[l][k] = sums[q];
            q++;
        }
    for (int k = 0; k < ND; k++) b[k] = sums[NT + k];
    const double tt = sums[NA - 1];
    bool ok = true;
    for (int k = 0; k < ND; k++) {
        const float g = d2f_rne(G[k][k]);
        sc[k] = (g > 0.f && g < 3.0e38f) ? f2d_exact(rsqrtf(g)) : 0.0;
    }
    for (int j = 0; j < ND && ok; j++) {
        double sjj = (sc[j] > 0.0 ? G[j][j] * sc[j] * sc[j] : 1.0) + 1e-12;
        for (int k = 0; k < j; k++) sjj -= L[j][k] * L[j][k];
        if (!(sjj > 0.0)) { ok = false; break; }
        rinv[j] = rsqrt_refined(sjj);
        L[j][j] = sjj * rinv[j];
        for (int i = j + 1; i < ND; i++) {
            double sij = G[i][j] * sc[i] * sc[j];
            for (int k = 0; k < j; k++) sij -= L[i][k] * L[j][k];
            L[i][j] = sij * rinv[j];
        }
    }
    if (ok) {
        for (int i = 0; i < ND; i++) {
            double r = b[i] * sc[i];
            for (int k = 0; k < i; k++) r -= L[i][k] * y[k];
            y[i] = r * rinv[i];
        }
        for (int i = ND - 1; i >= 0; i--) {
            double r = y[i];
            for (int k = i + 1; k < ND; k++) r -= L[k][i] * c[k];
            c[i] = r * rinv[i];
        }
        for (int i = 0; i < ND; i++) {
            c[i] *= sc[i];
            if (!isfinite(c[i])) ok = false;
        }
    }
    // misfit |t - D c|^2 = |t|^2 - 2 c.b + c^T G c; keep the fit only below
    // the unfitted change
    double mis = tt;
    if (ok) {
        for (int k = 0; k < ND; k++) {
            double gc = 0.0;
            for (int l = 0; l < ND; l++) gc += G[k][l] * c[l];
            mis += c[k] * (gc - 2.0 * b[k]);
        }
        if (!(mis <= tt)) ok = false;
    }
    double wa = 1.0;
    for (int k = 0; k < HIST_ND; k++) {
        const double ck = (ok && k < ND) ? c[k] : 0.0;
        F.coef[k] = ck;
        F.w[1 + k] = d_split(ck);
        wa -= ck;
    }
    F.w[0] = d_split(wa);
    // the misfit ratio (a diagnostic) in binary32
    const float tf = d2f_rne(tt), mf = d2f_rne(ok ? mis : tt);
    F.coef[HIST_ND] = tf > 0.f ? f2d_exact(sqrtf(fmaxf(mf, 0.f) / tf)) : 0.0;
}

}  // namespace qd
