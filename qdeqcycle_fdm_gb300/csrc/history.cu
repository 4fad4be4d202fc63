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
// Device data: a ring of m level-0 fields (the last m solutions, N x P
// each) stored as double-float pairs (d_split: hi + lo within 2^-47 of the
// FP64 value, 8 bytes a node like FP64), and their boundary columns in FP64
// packed as [fault rows 0..N-1, far rows 0..N-1].  Sixteen CTAs form the
// normal equations of the fit (at most 7 unknowns; one boundary value per
// thread, so that the strided loads of the boundary columns overlap); the
// last one scales them to a unit diagonal, adds a 1e-12 ridge, solves by
// Cholesky, keeps the fit only if its misfit is below the unfitted change
// and stores the weights as double-float pairs too; a grid then writes the
// guess into the interior columns as the weighted sum of the stored fields,
// evaluated in double-float arithmetic on the FP32 pipe (df_acc) with one
// FP64 addition per node to form the result.  In FP64 arithmetic the sum
// took ND + 1 fused multiply-adds per node on GB300's FP64 pipe (about one
// per SM clock), which bounded the kernel; the guess's rounding is now
// near 2^-46 of u instead of 2^-53, three orders of magnitude below what
// the solver's tolerances resolve.  Both kernels use programmatic dependent
// launch.  (One CTA of 512 threads, four values per thread and no cross-CTA
// hand-off, measured 8 us slower for the fit.)
#include <math.h>

#include <algorithm>

#include "hist_fit.cuh"

namespace qd {

struct History {
    int m = 0;          // capacity (0: off)
    int n = 0;          // stored solutions
    int head = 0;       // next slot to write
    size_t field = 0;   // nodes per stored field (N * P)
    float2 *u = nullptr;       // m fields (double-float pairs)
    double *bc = nullptr;      // m x 2N boundary values
    double *coef = nullptr;    // [HIST_ND] fit coefficients, [HIST_ND] misfit / change
    float2 *w = nullptr;       // [HIST_MAX] the guess's weights: the anchor's, then the coefficients
    double *partial = nullptr; // block sums of the fit: FIT_NA_MAX per block of the larger fit grid
    unsigned *count = nullptr; // CTAs of the fit done
    long long guesses = 0;
};

static History *hist(qd_solver *s) { return static_cast<History *>(s->history); }

__device__ __forceinline__ double bc_of(const double *u, int i, int N, int K, int P) {
    return i < N ? u[(long)i * P] : u[(long)(i - N) * P + K - 1];
}

// Normal equations of the fit over the 2N boundary values of u (one per
// thread, grid-stride), reduced and solved by fit_reduce_solve.
template <int ND>
__global__ void __launch_bounds__(FIT_THREADS) k_hist_fit(FitArgs F) {
    pdl_trigger();
    pdl_wait();
    FitAcc<ND> acc;
    acc.zero();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * F.N; i += gridDim.x * blockDim.x)
        acc.add(F, i, bc_of(F.u, i, F.N, F.K, F.P));
    fit_reduce_solve<ND>(F, acc);
}

struct ApplyArgs {
    double *u;
    const float2 *ring;
    size_t field;
    int N, K, P, a;
    int oth[HIST_ND];
    const float2 *w;
    double *implied;      // nullable: the combination's boundary values (2N)
};

// u = (1 - sum c_k) A + sum_k c_k S_k on the interior columns 1..K-2, in
// double-float arithmetic; the boundary columns keep the new data (their
// combination goes to `implied`).  One row per blockIdx.y, two nodes per
// thread.
template <int ND>
__global__ void k_hist_apply(ApplyArgs A) {
    pdl_wait();
    const int row = blockIdx.y, col = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (col >= A.K) return;
    float2 w[ND + 1];
#pragma unroll
    for (int k = 0; k <= ND; k++) w[k] = A.w[k];
    const size_t e = (size_t)row * A.P + col;
    float s0 = 0.f, l0 = 0.f, s1 = 0.f, l1 = 0.f;
    {
        const float4 av = __ldcs(reinterpret_cast<const float4 *>(A.ring + (size_t)A.a * A.field + e));
        df_acc(w[0].x, w[0].y, av.x, av.y, s0, l0);
        df_acc(w[0].x, w[0].y, av.z, av.w, s1, l1);
    }
#pragma unroll
    for (int k = 0; k < ND; k++) {
        const float4 sk = __ldcs(reinterpret_cast<const float4 *>(A.ring + (size_t)A.oth[k] * A.field + e));
        df_acc(w[k + 1].x, w[k + 1].y, sk.x, sk.y, s0, l0);
        df_acc(w[k + 1].x, w[k + 1].y, sk.z, sk.w, s1, l1);
    }
    const double2 v = make_double2(f2d_exact(s0) + f2d_exact(l0), f2d_exact(s1) + f2d_exact(l1));
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

// a stored field back into u (hi + lo, one FP64 addition per node)
__global__ void k_ring_to_u(const float2 *src, double *u, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float2 x = src[i];
        u[i] = f2d_exact(x.x) + f2d_exact(x.y);
    }
}

void history_free(qd_solver *s) {
    History *H = hist(s);
    if (!H) return;
    cudaFree(H->u);
    cudaFree(H->bc);
    cudaFree(H->coef);
    cudaFree(H->w);
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
    if (cudaMalloc(&H->u, sizeof(float2) * H->field * m) != cudaSuccess ||
        cudaMalloc(&H->bc, sizeof(double) * 2 * (size_t)d.N * m) != cudaSuccess ||
        cudaMalloc(&H->coef, sizeof(double) * (HIST_ND + 1)) != cudaSuccess ||
        cudaMalloc(&H->w, sizeof(float2) * HIST_MAX) != cudaSuccess ||
        cudaMalloc(&H->partial, sizeof(double) * std::max(FIT_CTAS, (d.N + FIT_THREADS - 1) / FIT_THREADS) *
                                    FIT_NA_MAX) != cudaSuccess ||
        cudaMalloc(&H->count, sizeof(unsigned)) != cudaSuccess) {
        (void)cudaGetLastError();
        history_free(s);
        set_error("solution history: out of device memory (%d fields of %zu doubles)", m, (size_t)d.N * d.P);
        return QD_ERR_CUDA;
    }
    QD_CUDA(cudaMemset(H->coef, 0, sizeof(double) * (HIST_ND + 1)));
    QD_CUDA(cudaMemset(H->w, 0, sizeof(float2) * HIST_MAX));
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

// the fit's arguments for anchor a and the other stored solutions
// oth[0..nd) (the boundary data of u when the fit reads them from u)
static FitArgs fit_args(qd_solver *s, History *H, int a, const int *oth, int nd) {
    const LevelDims &d = s->dims[0];
    FitArgs F{};
    F.u = s->L64[0].u;
    F.bc = H->bc;
    F.N = d.N; F.K = d.K; F.P = d.P;
    F.a = a;
    for (int k = 0; k < HIST_ND; k++) F.oth[k] = k < nd ? oth[k] : 0;
    F.coef = H->coef;
    F.w = H->w;
    F.partial = H->partial;
    F.count = H->count;
    return F;
}

// the guess the last fit gives, from anchor a and oth[0..nd), into u's
// interior
static int apply_from(qd_solver *s, History *H, int a, const int *oth, int nd, double *implied_bc) {
    const LevelDims &d = s->dims[0];
    ApplyArgs A{};
    A.u = s->L64[0].u;
    A.ring = H->u;
    A.field = H->field;
    A.N = d.N; A.K = d.K; A.P = d.P;
    A.a = a;
    for (int k = 0; k < HIST_ND; k++) A.oth[k] = k < nd ? oth[k] : 0;
    A.w = H->w;
    A.implied = implied_bc;
    const dim3 agrid((d.K + 255) / 256, d.N);
    switch (nd) {
#define QD_HIST_CASE(n)                                                                  \
    case n:                                                                              \
        QD_CUDA(launch_pdl(true, k_hist_apply<n>, agrid, dim3(128), 0, s->stream, A));   \
        break;
        QD_HIST_CASE(1) QD_HIST_CASE(2) QD_HIST_CASE(3) QD_HIST_CASE(4)
        QD_HIST_CASE(5) QD_HIST_CASE(6) QD_HIST_CASE(7)
#undef QD_HIST_CASE
        default:
            set_error("solution history: %d stored solutions", H->n);
            return QD_ERR_STATE;
    }
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

// the fit of the boundary data in u by the stored solutions a (anchor) and
// oth[0..nd) in a launch of its own (k_hist_fit), then the guess
static int guess_from(qd_solver *s, History *H, int a, const int *oth, int nd, double *implied_bc) {
    const FitArgs F = fit_args(s, H, a, oth, nd);
    const int fit_ctas = std::min(FIT_CTAS, (2 * s->dims[0].N + FIT_THREADS - 1) / FIT_THREADS);
    switch (nd) {
#define QD_HIST_CASE(n)                                                                                   \
    case n:                                                                                               \
        QD_CUDA(launch_pdl(true, k_hist_fit<n>, dim3(fit_ctas), dim3(FIT_THREADS), 0, s->stream, F));     \
        break;
        QD_HIST_CASE(1) QD_HIST_CASE(2) QD_HIST_CASE(3) QD_HIST_CASE(4)
        QD_HIST_CASE(5) QD_HIST_CASE(6) QD_HIST_CASE(7)
#undef QD_HIST_CASE
        default:
            set_error("solution history: %d stored solutions", H->n);
            return QD_ERR_STATE;
    }
    QD_LAUNCH_CHECK(s);
    return apply_from(s, H, a, oth, nd, implied_bc);
}

// The stage's fit, for launch_stage_boundary to carry out in the boundary
// kernel (the new boundary data come from that kernel's registers):
// returns the number of fit unknowns (0: the next solve starts from the
// previous solution, no fit) and fills *F.
int history_fit_args(qd_solver *s, FitArgs *F) {
    History *H = hist(s);
    if (!H || H->n < 2) return 0;
    int a, oth[HIST_ND];
    const int nd = history_slots(H, &a, oth);
    *F = fit_args(s, H, a, oth, nd);
    return nd;
}

// after the stage's boundary kernel fitted the new data: replace the
// interior by the fitted combination (no-op with fewer than two stored
// solutions)
int history_apply(qd_solver *s, double *implied_bc) {
    History *H = hist(s);
    if (!H || H->n < 2) return QD_OK;
    int a, oth[HIST_ND];
    const int nd = history_slots(H, &a, oth);
    QD_TRY(apply_from(s, H, a, oth, nd, implied_bc));
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
    const long n = (long)d.N * d.P;
    k_ring_to_u<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(H->u + (size_t)a * H->field, s->L64[0].u, n);
    QD_LAUNCH_CHECK(s);
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
