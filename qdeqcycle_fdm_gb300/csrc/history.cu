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
// 0..N-1].  One CTA forms the normal equations of the fit (at most 7
// unknowns), scales them to a unit diagonal, adds a 1e-12 ridge, solves by
// Cholesky and keeps the fit only if its misfit is below the unfitted
// change; a grid then writes the guess into the interior columns.
#include <math.h>

#include "qdeq_internal.cuh"

namespace qd {

static constexpr int HIST_MAX = 8;              // stored solutions
static constexpr int HIST_ND = HIST_MAX - 1;     // fit unknowns
static constexpr int HIST_NTRI = HIST_ND * (HIST_ND + 1) / 2;
static constexpr int HIST_NACC = HIST_NTRI + HIST_ND + 1;
static constexpr int HIST_THREADS = 512;

struct History {
    int m = 0;          // capacity (0: off)
    int n = 0;          // stored solutions
    int head = 0;       // next slot to write
    size_t field = 0;   // doubles per stored field (N * P)
    double *u = nullptr;     // m fields
    double *bc = nullptr;    // m x 2N boundary values
    double *coef = nullptr;  // [HIST_ND] fit coefficients, [HIST_ND] misfit / change
    long long guesses = 0;
};

static History *hist(qd_solver *s) { return static_cast<History *>(s->history); }

__device__ __forceinline__ double bc_of(const double *u, int i, int N, int K, int P) {
    return i < N ? u[(long)i * P] : u[(long)(i - N) * P + K - 1];
}

// packed index of G[k][l], k <= l
__host__ __device__ constexpr int tri(int k, int l) { return k * HIST_ND - k * (k - 1) / 2 + (l - k); }

// block-wide sum of v[0..n) into out[0..n) (every thread gets the sums)
template <int NV>
__device__ void block_sum(double (&v)[NV], int n, double (*red)[NV + 1], double *out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; i++) {
        if (i >= n) break;
        double x = v[i];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][i] = x;
    }
    __syncthreads();
    if (threadIdx.x < n) {
        double x = 0.0;
        for (int w = 0; w < nw; w++) x += red[w][threadIdx.x];   // fixed order: deterministic
        out[threadIdx.x] = x;
    }
    __syncthreads();
}

// anchor = slot a, the other stored solutions = slots oth[0..nd)
struct FitArgs {
    const double *u;      // the solver's u with the new boundary data in columns 0, K-1
    const double *bc;     // ring of boundary values
    int N, K, P, nd, a;
    int oth[HIST_ND];
    double *coef;
    double *implied;      // nullable: receives g_A + sum c_k (g_k - g_A) (2N values)
};

__global__ void __launch_bounds__(HIST_THREADS) k_hist_fit(FitArgs F) {
    __shared__ double red[HIST_THREADS / 32][HIST_NACC + 1];
    __shared__ double sums[HIST_NACC];
    __shared__ double c[HIST_ND];
    const int n2 = 2 * F.N, nd = F.nd;
    const double *gA = F.bc + (size_t)F.a * n2;

    // pass 1: G = D^T D (upper triangle), b = D^T t, |t|^2, packed at fixed
    // places for all HIST_ND unknowns (differences past nd are zero)
    double acc[HIST_NACC];
#pragma unroll
    for (int i = 0; i < HIST_NACC; i++) acc[i] = 0.0;
    for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const double ga = gA[i], t = bc_of(F.u, i, F.N, F.K, F.P) - ga;
        double d[HIST_ND];
#pragma unroll
        for (int k = 0; k < HIST_ND; k++) d[k] = k < nd ? F.bc[(size_t)F.oth[k] * n2 + i] - ga : 0.0;
#pragma unroll
        for (int k = 0; k < HIST_ND; k++)
#pragma unroll
            for (int l = k; l < HIST_ND; l++) acc[tri(k, l)] += d[k] * d[l];
#pragma unroll
        for (int k = 0; k < HIST_ND; k++) acc[HIST_NTRI + k] += d[k] * t;
        acc[HIST_NACC - 1] += t * t;
    }
    block_sum<HIST_NACC>(acc, HIST_NACC, red, sums);

    if (threadIdx.x == 0) {
        double G[HIST_ND][HIST_ND], b[HIST_ND], sc[HIST_ND], L[HIST_ND][HIST_ND], y[HIST_ND];
        for (int k = 0; k < nd; k++)
            for (int l = k; l < nd; l++) G[k][l] = G[l][k] = sums[tri(k, l)];
        for (int k = 0; k < nd; k++) b[k] = sums[HIST_NTRI + k];
        bool ok = true;
        for (int k = 0; k < nd; k++) sc[k] = G[k][k] > 0.0 ? 1.0 / sqrt(G[k][k]) : 0.0;
        for (int j = 0; j < nd && ok; j++) {
            double sjj = (sc[j] > 0.0 ? G[j][j] * sc[j] * sc[j] : 1.0) + 1e-12;
            for (int k = 0; k < j; k++) sjj -= L[j][k] * L[j][k];
            if (!(sjj > 0.0)) { ok = false; break; }
            L[j][j] = sqrt(sjj);
            for (int i = j + 1; i < nd; i++) {
                double sij = G[i][j] * sc[i] * sc[j];
                for (int k = 0; k < j; k++) sij -= L[i][k] * L[j][k];
                L[i][j] = sij / L[j][j];
            }
        }
        if (ok) {
            for (int i = 0; i < nd; i++) {
                double r = b[i] * sc[i];
                for (int k = 0; k < i; k++) r -= L[i][k] * y[k];
                y[i] = r / L[i][i];
            }
            for (int i = nd - 1; i >= 0; i--) {
                double r = y[i];
                for (int k = i + 1; k < nd; k++) r -= L[k][i] * c[k];
                c[i] = r / L[i][i];
            }
            for (int i = 0; i < nd; i++) {
                c[i] *= sc[i];
                if (!isfinite(c[i])) ok = false;
            }
        }
        if (!ok)
            for (int i = 0; i < nd; i++) c[i] = 0.0;
    }
    __syncthreads();

    // pass 2: misfit of the fit; keep it only below the unfitted change
    double mis[1] = {0.0};
    for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const double ga = gA[i];
        double r = bc_of(F.u, i, F.N, F.K, F.P) - ga;
        for (int k = 0; k < nd; k++) r -= c[k] * (F.bc[(size_t)F.oth[k] * n2 + i] - ga);
        mis[0] += r * r;
    }
    __shared__ double red1[HIST_THREADS / 32][2];
    __shared__ double msum[1];
    block_sum<1>(mis, 1, red1, msum);
    const double tt = sums[HIST_NACC - 1];
    const bool keep = msum[0] <= tt;
    if (threadIdx.x == 0) {
        for (int k = 0; k < HIST_ND; k++) F.coef[k] = (keep && k < nd) ? c[k] : 0.0;
        F.coef[HIST_ND] = tt > 0.0 ? sqrt((keep ? msum[0] : tt) / tt) : 0.0;
    }
    if (!keep) {
        __syncthreads();
        if (threadIdx.x < nd) c[threadIdx.x] = 0.0;
    }
    __syncthreads();
    if (F.implied)
        for (int i = threadIdx.x; i < n2; i += blockDim.x) {
            const double ga = gA[i];
            double v = ga;
            for (int k = 0; k < nd; k++) v += c[k] * (F.bc[(size_t)F.oth[k] * n2 + i] - ga);
            F.implied[i] = v;
        }
}

struct ApplyArgs {
    double *u;
    const double *ring;
    size_t field;
    int N, K, P, nd, a;
    int oth[HIST_ND];
    const double *coef;
};

// interior columns 1..K-2: u = A + sum_k c_k (S_k - A); two nodes per thread
__global__ void k_hist_apply(ApplyArgs A) {
    const long pairs = (long)A.N * A.P / 2;
    double c[HIST_ND];
#pragma unroll
    for (int k = 0; k < HIST_ND; k++) c[k] = k < A.nd ? A.coef[k] : 0.0;
    const double *Ua = A.ring + (size_t)A.a * A.field;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < pairs; q += (long)gridDim.x * blockDim.x) {
        const long e = 2 * q;
        const int col = (int)(e % A.P);
        if (col >= A.K) continue;
        const double2 av = __ldcs(reinterpret_cast<const double2 *>(Ua + e));
        double2 v = av;
#pragma unroll
        for (int k = 0; k < HIST_ND; k++) {
            if (k >= A.nd) break;
            const double2 sk = __ldcs(reinterpret_cast<const double2 *>(A.ring + (size_t)A.oth[k] * A.field + e));
            v.x += c[k] * (sk.x - av.x);
            v.y += c[k] * (sk.y - av.y);
        }
        double2 *dst = reinterpret_cast<double2 *>(A.u + e);
        double2 o = *dst;                       // columns 0 and K-1 keep the new boundary data
        if (col >= 1 && col <= A.K - 2) o.x = v.x;
        if (col + 1 >= 1 && col + 1 <= A.K - 2) o.y = v.y;
        *dst = o;
    }
}

// copy the solved u into ring slot `slot` and pack its boundary columns
__global__ void k_hist_push(const double *u, double *dst, double *bc, size_t field, int N, int K, int P) {
    const long pairs = (long)field / 2;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < pairs; q += (long)gridDim.x * blockDim.x) {
        const double2 v = reinterpret_cast<const double2 *>(u)[q];
        reinterpret_cast<double2 *>(dst)[q] = v;
        const long e = 2 * q;
        const int row = (int)(e / P), col = (int)(e - (long)row * P);
        if (col == 0) bc[row] = v.x;
        if (col == K - 2) bc[N + row] = v.y;
        if (col == K - 1) bc[N + row] = v.x;
    }
}

static int stream_grid(long items) {
    long g = (items + 255) / 256;
    const long cap = 152L * 8;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

void history_free(qd_solver *s) {
    History *H = hist(s);
    if (!H) return;
    cudaFree(H->u);
    cudaFree(H->bc);
    cudaFree(H->coef);
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
        cudaMalloc(&H->coef, sizeof(double) * (HIST_ND + 1)) != cudaSuccess) {
        (void)cudaGetLastError();
        history_free(s);
        set_error("solution history: out of device memory (%d fields of %zu doubles)", m, (size_t)d.N * d.P);
        return QD_ERR_CUDA;
    }
    QD_CUDA(cudaMemset(H->coef, 0, sizeof(double) * (HIST_ND + 1)));
    return QD_OK;
}

// slots of the anchor (latest) and of the other stored solutions, newest first
static int history_slots(const History *H, int *a, int oth[HIST_ND]) {
    *a = (H->head - 1 + H->m) % H->m;
    const int nd = H->n - 1;
    for (int k = 0; k < nd; k++) oth[k] = (H->head - 2 - k + 2 * H->m) % H->m;
    return nd;
}

// after the stage's boundary data are in u: replace the interior by the
// fitted combination (no-op with fewer than two stored solutions)
int history_guess(qd_solver *s, double *implied_bc) {
    History *H = hist(s);
    if (!H || H->n < 2) return QD_OK;
    const LevelDims &d = s->dims[0];
    FitArgs F{};
    F.u = s->L64[0].u;
    F.bc = H->bc;
    F.N = d.N; F.K = d.K; F.P = d.P;
    F.nd = history_slots(H, &F.a, F.oth);
    F.coef = H->coef;
    F.implied = implied_bc;
    k_hist_fit<<<1, HIST_THREADS, 0, s->stream>>>(F);
    QD_LAUNCH_CHECK(s);
    ApplyArgs A{};
    A.u = s->L64[0].u;
    A.ring = H->u;
    A.field = H->field;
    A.N = d.N; A.K = d.K; A.P = d.P;
    A.nd = F.nd; A.a = F.a;
    for (int k = 0; k < HIST_ND; k++) A.oth[k] = F.oth[k];
    A.coef = H->coef;
    k_hist_apply<<<stream_grid((long)H->field / 2), 256, 0, s->stream>>>(A);
    QD_LAUNCH_CHECK(s);
    H->guesses++;
    return QD_OK;
}

// after a stage solve: store the solution
int history_push(qd_solver *s) {
    History *H = hist(s);
    if (!H) return QD_OK;
    const LevelDims &d = s->dims[0];
    const int slot = H->head;
    k_hist_push<<<stream_grid((long)H->field / 2), 256, 0, s->stream>>>(
        s->L64[0].u, H->u + (size_t)slot * H->field, H->bc + (size_t)slot * 2 * d.N, H->field, d.N, d.K, d.P);
    QD_LAUNCH_CHECK(s);
    H->head = (H->head + 1) % H->m;
    if (H->n < H->m) H->n++;
    return QD_OK;
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
