// history.cu -- warm start of the stage solves from the solution history.
//
// Every stage solve of the RK43 driver solves the same operator with new
// Dirichlet data on two columns: the fault (slip/2, odeSolver.cpp:1160) and
// the far boundary (Vp (t + c dt)/2 + shift, :1170).  The interior of a
// converged solution is the discrete harmonic extension of its boundary
// data, so a linear combination of earlier solutions is the harmonic
// extension of the same combination of their boundary data.  The guess
//
//   u = A + sum_k c_k (S_k - A)      (A: the latest solution, S_k: earlier ones)
//
// with c the least-squares fit of the new boundary data g by those of the
// stored solutions,  min_c || (g - g_A) - sum_k c_k (g_k - g_A) ||_2,  has an
// initial error equal to the harmonic extension of the fit's misfit instead
// of that of the whole change g - g_A (the reference starts every solve from
// the previous solution, c = 0).  The boundary data of successive stages lie
// close to the span of the last few, so the misfit is orders of magnitude
// below the change and the solve needs fewer V-cycles to reach the same
// tolerance.  Only the starting point moves; the multigrid still iterates to
// the solver's residual tolerance.
//
// Device data: a ring of m level-0 FP64 fields (the last m solutions, N x P
// each) and their boundary columns packed as [fault rows 0..N-1, far rows
// 0..N-1].  Sixteen CTAs form the normal equations of the fit (at most 7
// unknowns; one boundary value per thread, so that the strided loads of the
// boundary columns overlap); the last one scales them to a unit diagonal,
// adds a 1e-12 ridge, solves by Cholesky and keeps the fit only if its
// misfit is below the unfitted change; a grid then writes the guess into
// the interior columns as a weighted sum of the stored fields.  Both
// kernels use programmatic dependent launch.  (One CTA of 512 threads, four
// values per thread and no cross-CTA hand-off, measured 8 us slower.)
#include <math.h>

#include <algorithm>

#include "qdeq_internal.cuh"

namespace qd {

static constexpr int HIST_MAX = 8;              // stored solutions
static constexpr int HIST_ND = HIST_MAX - 1;     // fit unknowns at most
static constexpr int FIT_THREADS = 128;
static constexpr int FIT_CTAS = 16;
static constexpr int FIT_NA_MAX = HIST_ND * (HIST_ND + 1) / 2 + HIST_ND + 1;

struct History {
    int m = 0;          // capacity (0: off)
    int n = 0;          // stored solutions
    int head = 0;       // next slot to write
    size_t field = 0;   // doubles per stored field (N * P)
    double *u = nullptr;       // m fields
    double *bc = nullptr;      // m x 2N boundary values
    double *coef = nullptr;    // [HIST_ND] fit coefficients, [HIST_ND] misfit / change
    double *partial = nullptr; // FIT_CTAS x FIT_NA_MAX block sums of the fit
    unsigned *count = nullptr; // CTAs of the fit done
    long long guesses = 0;
};

static History *hist(qd_solver *s) { return static_cast<History *>(s->history); }

__device__ __forceinline__ double bc_of(const double *u, int i, int N, int K, int P) {
    return i < N ? u[(long)i * P] : u[(long)(i - N) * P + K - 1];
}

// anchor = slot a, the other stored solutions = slots oth[0..nd)
struct FitArgs {
    const double *u;      // the solver's u with the new boundary data in columns 0, K-1
    const double *bc;     // ring of boundary values
    int N, K, P, a;
    int oth[HIST_ND];
    double *coef, *partial;
    unsigned *count;
};

// Normal equations of the fit over the 2N boundary values; with more than
// one block the last block to finish sums the block partials in a fixed
// order (deterministic) and solves.  Accumulators per boundary value:
// G = D^T D (upper triangle), b = D^T t, |t|^2.
template <int ND>
__global__ void __launch_bounds__(FIT_THREADS) k_hist_fit(FitArgs F) {
    pdl_trigger();
    pdl_wait();
    constexpr int NT = ND * (ND + 1) / 2, NA = NT + ND + 1;
    __shared__ double red[FIT_THREADS / 32][NA];
    __shared__ double sums[NA];
    __shared__ int is_last;
    const int n2 = 2 * F.N, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double *gA = F.bc + (size_t)F.a * n2;

    double acc[NA];
#pragma unroll
    for (int i = 0; i < NA; i++) acc[i] = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        const double ga = gA[i], t = bc_of(F.u, i, F.N, F.K, F.P) - ga;
        double d[ND];
#pragma unroll
        for (int k = 0; k < ND; k++) d[k] = F.bc[(size_t)F.oth[k] * n2 + i] - ga;
        int q = 0;
#pragma unroll
        for (int k = 0; k < ND; k++)
#pragma unroll
            for (int l = k; l < ND; l++) acc[q++] += d[k] * d[l];
#pragma unroll
        for (int k = 0; k < ND; k++) acc[NT + k] += d[k] * t;
        acc[NA - 1] += t * t;
    }
#pragma unroll
    for (int i = 0; i < NA; i++) {
        double x = acc[i];
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

    // unit-diagonal scaling, 1e-12 ridge, Cholesky
    double G[ND][ND], b[ND], sc[ND], L[ND][ND], y[ND], c[ND];
    int q = 0;
    for (int k = 0; k < ND; k++)
        for (int l = k; l < ND; l++) {
            G[k][l] = G[l][k] = sums[q];
            q++;
        }
    for (int k = 0; k < ND; k++) b[k] = sums[NT + k];
    const double tt = sums[NA - 1];
    bool ok = true;
    for (int k = 0; k < ND; k++) sc[k] = G[k][k] > 0.0 ? 1.0 / sqrt(G[k][k]) : 0.0;
    for (int j = 0; j < ND && ok; j++) {
        double sjj = (sc[j] > 0.0 ? G[j][j] * sc[j] * sc[j] : 1.0) + 1e-12;
        for (int k = 0; k < j; k++) sjj -= L[j][k] * L[j][k];
        if (!(sjj > 0.0)) { ok = false; break; }
        L[j][j] = sqrt(sjj);
        for (int i = j + 1; i < ND; i++) {
            double sij = G[i][j] * sc[i] * sc[j];
            for (int k = 0; k < j; k++) sij -= L[i][k] * L[j][k];
            L[i][j] = sij / L[j][j];
        }
    }
    if (ok) {
        for (int i = 0; i < ND; i++) {
            double r = b[i] * sc[i];
            for (int k = 0; k < i; k++) r -= L[i][k] * y[k];
            y[i] = r / L[i][i];
        }
        for (int i = ND - 1; i >= 0; i--) {
            double r = y[i];
            for (int k = i + 1; k < ND; k++) r -= L[k][i] * c[k];
            c[i] = r / L[i][i];
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
    for (int k = 0; k < HIST_ND; k++) F.coef[k] = (ok && k < ND) ? c[k] : 0.0;
    F.coef[HIST_ND] = tt > 0.0 ? sqrt(fmax(ok ? mis : tt, 0.0) / tt) : 0.0;
}

struct ApplyArgs {
    double *u;
    const double *ring;
    size_t field;
    int N, K, P, a;
    int oth[HIST_ND];
    const double *coef;
    double *implied;      // nullable: the combination's boundary values (2N)
};

// u = (1 - sum c_k) A + sum_k c_k S_k on the interior columns 1..K-2; the
// boundary columns keep the new data (their combination goes to `implied`).
// One row per blockIdx.y, two nodes per thread.
template <int ND>
__global__ void k_hist_apply(ApplyArgs A) {
    pdl_wait();
    const int row = blockIdx.y, col = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (col >= A.K) return;
    double c[ND], wa = 1.0;
#pragma unroll
    for (int k = 0; k < ND; k++) {
        c[k] = A.coef[k];
        wa -= c[k];
    }
    const size_t e = (size_t)row * A.P + col;
    const double2 av = __ldcs(reinterpret_cast<const double2 *>(A.ring + (size_t)A.a * A.field + e));
    double2 v = make_double2(wa * av.x, wa * av.y);
#pragma unroll
    for (int k = 0; k < ND; k++) {
        const double2 sk = __ldcs(reinterpret_cast<const double2 *>(A.ring + (size_t)A.oth[k] * A.field + e));
        v.x = fma(c[k], sk.x, v.x);
        v.y = fma(c[k], sk.y, v.y);
    }
    double2 *dst = reinterpret_cast<double2 *>(A.u + e);
    // only a pair holding a boundary column (or the padding) keeps part of u
    double2 o = (col >= 1 && col + 1 <= A.K - 2) ? v : *dst;
    if (col >= 1 && col <= A.K - 2) o.x = v.x;
    if (col + 1 <= A.K - 2) o.y = v.y;
    *dst = o;
    if (A.implied) {
        if (col == 0) A.implied[row] = v.x;
        if (col == A.K - 1) A.implied[A.N + row] = v.x;
        if (col + 1 == A.K - 1) A.implied[A.N + row] = v.y;
    }
}

void history_free(qd_solver *s) {
    History *H = hist(s);
    if (!H) return;
    cudaFree(H->u);
    cudaFree(H->bc);
    cudaFree(H->coef);
    cudaFree(H->partial);
    cudaFree(H->count);
    delete H;
    s->history = nullptr;
}

void history_reset(qd_solver *s) {
    if (History *H = hist(s)) {
        H->n = 0;
        H->head = 0;
    }
}

int history_set(qd_solver *s, int m) {
    if (m < 0 || m > HIST_MAX) {
        set_error("solution history: m must be 0..%d", HIST_MAX);
        return QD_ERR_ARG;
    }
    QD_CUDA(cudaStreamSynchronize(s->stream));
    history_free(s);
    if (m < 2) return QD_OK;              // 0 or 1: start from the previous solution
    const LevelDims &d = s->dims[0];
    History *H = new History();
    H->m = m;
    H->field = (size_t)d.N * d.P;
    s->history = H;
    if (cudaMalloc(&H->u, sizeof(double) * H->field * m) != cudaSuccess ||
        cudaMalloc(&H->bc, sizeof(double) * 2 * (size_t)d.N * m) != cudaSuccess ||
        cudaMalloc(&H->coef, sizeof(double) * (HIST_ND + 1)) != cudaSuccess ||
        cudaMalloc(&H->partial, sizeof(double) * FIT_CTAS * FIT_NA_MAX) != cudaSuccess ||
        cudaMalloc(&H->count, sizeof(unsigned)) != cudaSuccess) {
        (void)cudaGetLastError();
        history_free(s);
        set_error("solution history: out of device memory (%d fields of %zu doubles)", m, (size_t)d.N * d.P);
        return QD_ERR_CUDA;
    }
    QD_CUDA(cudaMemset(H->coef, 0, sizeof(double) * (HIST_ND + 1)));
    QD_CUDA(cudaMemset(H->count, 0, sizeof(unsigned)));
    return QD_OK;
}

// slots of the anchor (latest) and of the other stored solutions, newest first
static int history_slots(const History *H, int *a, int oth[HIST_ND]) {
    *a = (H->head - 1 + H->m) % H->m;
    const int nd = H->n - 1;
    for (int k = 0; k < nd; k++) oth[k] = (H->head - 2 - k + 2 * H->m) % H->m;
    return nd;
}

// the fit of the boundary data in u by the stored solutions a (anchor) and
// oth[0..nd), and the guess it gives in u's interior
static int guess_from(qd_solver *s, History *H, int a, const int *oth, int nd, double *implied_bc) {
    const LevelDims &d = s->dims[0];
    FitArgs F{};
    F.u = s->L64[0].u;
    F.bc = H->bc;
    F.N = d.N; F.K = d.K; F.P = d.P;
    F.a = a;
    for (int k = 0; k < HIST_ND; k++) F.oth[k] = k < nd ? oth[k] : 0;
    F.coef = H->coef;
    F.partial = H->partial;
    F.count = H->count;
    ApplyArgs A{};
    A.u = s->L64[0].u;
    A.ring = H->u;
    A.field = H->field;
    A.N = d.N; A.K = d.K; A.P = d.P;
    A.a = F.a;
    for (int k = 0; k < HIST_ND; k++) A.oth[k] = F.oth[k];
    A.coef = H->coef;
    A.implied = implied_bc;
    const int fit_ctas = std::min(FIT_CTAS, (2 * d.N + FIT_THREADS - 1) / FIT_THREADS);
    const dim3 agrid((d.K + 255) / 256, d.N);
    switch (nd) {
#define QD_HIST_CASE(n)                                                       \
    case n:                                                                   \
        QD_CUDA(launch_pdl(true, k_hist_fit<n>, dim3(fit_ctas), dim3(FIT_THREADS), 0, s->stream, F)); \
        QD_LAUNCH_CHECK(s);                                                   \
        QD_CUDA(launch_pdl(true, k_hist_apply<n>, agrid, dim3(128), 0, s->stream, A)); \
        QD_LAUNCH_CHECK(s);                                                   \
        break;
        QD_HIST_CASE(1) QD_HIST_CASE(2) QD_HIST_CASE(3) QD_HIST_CASE(4)
        QD_HIST_CASE(5) QD_HIST_CASE(6) QD_HIST_CASE(7)
#undef QD_HIST_CASE
        default:
            set_error("solution history: %d stored solutions", H->n);
            return QD_ERR_STATE;
    }
    return QD_OK;
}

// after the stage's boundary data are in u: replace the interior by the
// fitted combination (no-op with fewer than two stored solutions)
int history_guess(qd_solver *s, double *implied_bc) {
    History *H = hist(s);
    if (!H || H->n < 2) return QD_OK;
    int a, oth[HIST_ND];
    const int nd = history_slots(H, &a, oth);
    QD_TRY(guess_from(s, H, a, oth, nd, implied_bc));
    H->guesses++;
    return QD_OK;
}

// The last stored solve once more: u = the newest stored solution (its
// boundary data and, as the answer, its interior), then the guess the
// other stored solutions give for it, as the solve had started from with
// one stored solution fewer.  The ring is left as it is.  QD_ERR_STATE
// with fewer than three stored solutions.
int history_replay_guess(qd_solver *s) {
    History *H = hist(s);
    if (!H || H->n < 3) return QD_ERR_STATE;
    int a, oth[HIST_ND];
    const int nd = history_slots(H, &a, oth);
    const LevelDims &d = s->dims[0];
    QD_CUDA(cudaMemcpyAsync(s->L64[0].u, H->u + (size_t)a * H->field, sizeof(double) * (size_t)d.N * d.P,
                            cudaMemcpyDeviceToDevice, s->stream));
    return guess_from(s, H, oth[0], oth + 1, nd - 1, nullptr);
}

// after a stage solve: the copy of the solution into the ring, for the
// fault stage's launch to carry out (launch_fault)
int history_push_job(qd_solver *s, CopyJob *job) {
    *job = CopyJob{};
    History *H = hist(s);
    if (!H) return QD_OK;
    const LevelDims &d = s->dims[0];
    const int slot = H->head;
    job->src = s->L64[0].u;
    job->dst = H->u + (size_t)slot * H->field;
    job->bc = H->bc + (size_t)slot * 2 * d.N;
    job->N = d.N;
    job->K = d.K;
    job->P = d.P;
    H->head = (H->head + 1) % H->m;
    if (H->n < H->m) H->n++;
    return QD_OK;
}

// true when the next stage solve will start from a fitted guess
bool history_will_guess(qd_solver *s) {
    const History *H = hist(s);
    return H && H->n >= 2;
}

// host copy of the last fit: coefficients [HIST_ND] and the misfit ratio
int history_last_fit(qd_solver *s, double *out, int *nd) {
    History *H = hist(s);
    if (!H) {
        *nd = 0;
        return QD_OK;
    }
    QD_CUDA(cudaMemcpyAsync(out, H->coef, sizeof(double) * (HIST_ND + 1), cudaMemcpyDeviceToHost, s->stream));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    *nd = H->n > 0 ? H->n - 1 : 0;
    return QD_OK;
}

}  // namespace qd
