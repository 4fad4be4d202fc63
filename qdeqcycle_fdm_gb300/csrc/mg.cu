// mg.cu -- geometric multigrid for  div(mu grad u) = f  on the fault-normal
// plane, FP64 and FP32, on one GB300.
//
// What is solved is exactly the reference's discrete problem
// (odeSolver.cpp:757-1147):
//   * 5-point variable-coefficient operator, Dirichlet columns 0 and K-1,
//     mirrored (Neumann) first and last rows;
//   * level-0 face moduli from mu_equi's half-grid edges; coarse levels use
//     the node modulus half-way between coarse nodes (fin_coa indexing,
//     :823-827), and on coarse levels the mirrored rows take the inner face
//     twice (:830-847) -- folded here into cz[0] = cz[1], cz[N] = cz[N-1];
//   * red-black Gauss-Seidel with relaxation 1, red = (j+k) even first;
//   * full-weighting restriction with mirrored rows (:953-1015) and bilinear
//     prolongation that skips the last fine row (:1017-1043);
//   * V-cycle recursion with smoothing only on the coarsest level.
// The smoother multiplies by a precomputed 1/diag (the reference divides
// 1/diag on the fly); red-black order makes each colour update independent
// of thread order, so results are deterministic.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <vector>

#include "qdeq_internal.cuh"

namespace qd {

static constexpr int BX = 32, BY = 8;

__host__ __device__ static inline int cdiv(int a, int b) { return (a + b - 1) / b; }

template <typename T>
struct View {
    T *u;
    const T *f;
    T *r;
    const T *cx, *cz, *dinv;
    int N, K, P;
    T h2, inv_h2;
};

template <typename T>
static View<T> make_view(const qd_solver *s, const Level<T> *Ls, int l) {
    View<T> v;
    v.u = Ls[l].u; v.f = Ls[l].f; v.r = Ls[l].r;
    v.cx = Ls[l].cx; v.cz = Ls[l].cz; v.dinv = Ls[l].dinv;
    v.N = s->dims[l].N; v.K = s->dims[l].K; v.P = s->dims[l].P;
    v.h2 = (T)s->dims[l].h2; v.inv_h2 = (T)s->dims[l].inv_h2;
    return v;
}

// ---------------------------------------------------------------------------
// reductions (deterministic: fixed block shape, fixed tree)
// ---------------------------------------------------------------------------
__device__ static double block_sum(double v) {
    __shared__ double sh[32];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nthr = blockDim.x * blockDim.y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) sh[tid >> 5] = v;
    __syncthreads();
    if (tid < 32) {
        v = (tid < (nthr + 31) / 32) ? sh[tid] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;  // valid in thread 0
}

// block_sum in binary32 (valid in thread 0)
__device__ static float block_sum_f(float v) {
    __shared__ float sh[32];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nthr = blockDim.x * blockDim.y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) sh[tid >> 5] = v;
    __syncthreads();
    if (tid < 32) {
        v = (tid < (nthr + 31) / 32) ? sh[tid] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;
}

// block_sum of double-float pairs (valid in thread 0)
__device__ static float2 block_sum_df(float2 v) {
    __shared__ float2 sh[32];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nthr = blockDim.x * blockDim.y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = df_add(v, make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o)));
    if ((tid & 31) == 0) sh[tid >> 5] = v;
    __syncthreads();
    if (tid < 32) {
        v = (tid < (nthr + 31) / 32) ? sh[tid] : make_float2(0.f, 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v = df_add(v, make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o)));
    }
    __syncthreads();
    return v;
}

__global__ void k_final_sum(const double *partial, int n, double *out) {
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += partial[i];
    v = block_sum(v);
    if (threadIdx.x == 0) *out = v;
}

// ---------------------------------------------------------------------------
// coefficient set-up from the reference's staggered mu_equi
//
// With a depth metric (a grid stretched in depth, z = z(zeta) on a uniform
// computational coordinate zeta of spacing dh), the operator is
//   J d/dx(mu du/dx) + d/dzeta((mu / J) du/dzeta),   J = dz/dzeta,
// the conservative form of div(mu grad u) multiplied by J: the same 5-point
// stencil on the uniform (x, zeta) grid with x-face moduli mu J (J at the
// face's row) and z-face moduli mu / J (J at the face).  jrow holds J per
// staggered row of mu_equi (node rows even, face rows odd, the ghost rows
// mirrored), so each coefficient takes the metric of the mu_equi row it is
// read from; null: the reference's uniform grid.
// ---------------------------------------------------------------------------
__global__ void k_build_faces(const double *__restrict__ mu, const double *__restrict__ jrow, long W,
                              int level, int fc, int N, int K, int P, double *cx, double *cz) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (k >= K || j > N) return;
    if (j < N && k < K - 1) {
        long row, col;
        if (level == 0) {
            col = (k + 1) * 2 + 1; row = (long)(j + 1) * 2;                    // index2, :787
        } else {
            col = ((k * 2 + 1) * fc / 2 + 1) * 2; row = (long)(j * fc + 1) * 2;  // :825
        }
        const double m = mu[col + row * W];
        cx[(long)j * P + k] = jrow ? m * jrow[row] : m;
    }
    long row;
    if (level == 0) {
        row = 2 * j + 1;                                                  // index3 of row j, :788
    } else {
        const int jj = (j == 0) ? 1 : (j == N ? N - 1 : j);                // :830-847 quirk
        row = (long)((jj * 2 - 1) * fc / 2 + 1) * 2;                      // :826
    }
    const double m = mu[(k * fc + 1) * 2 + row * W];
    cz[(long)j * P + k] = jrow ? m / jrow[row] : m;
}

__global__ void k_build_dinv(int N, int K, int P, const double *cx, const double *cz,
                             double *dinv, float *cx32, float *cz32, float *dinv32, double *diag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (k >= K || j > N) return;
    const long c = (long)j * P + k;
    cz32[c] = (float)cz[c];
    if (j == N) return;
    if (k < K - 1) cx32[c] = (float)cx[c];
    if (k >= 1 && k <= K - 2) {
        // relax_rbgs / (mu1 + mu2 + mu3 + mu4), same summation order (:794-795)
        const double sum = ((cx[c - 1] + cx[c]) + cz[c]) + cz[c + P];
        const double d = 1.00 / sum;
        dinv[c] = d;
        dinv32[c] = (float)d;
        if (diag) diag[c] = sum;
    }
}

// ---------------------------------------------------------------------------
// smoother: one colour of red-black Gauss-Seidel, one thread per node of the
// colour (the reference launches one thread per node and idles half).
// ---------------------------------------------------------------------------
template <typename T, bool HAS_F>
__global__ void __launch_bounds__(BX * BY) k_rb(View<T> v, int color) {
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= v.N) return;
    const int k = 2 * kk + 1 + ((j + 1 + color) & 1);
    if (k > v.K - 2) return;
    const long c = (long)j * v.P + k;
    const long up = (j == 0) ? v.P : -(long)v.P;          // row j-1 (mirrored at j = 0)
    const long dn = (j == v.N - 1) ? -(long)v.P : v.P;    // row j+1 (mirrored at j = N-1)
    const T *u = v.u;
    T acc = v.cx[c - 1] * u[c - 1] + v.cx[c] * u[c + 1] + v.cz[c] * u[c + up] +
            v.cz[c + v.P] * u[c + dn];
    if (HAS_F) acc -= v.h2 * v.f[c];
    v.u[c] = v.dinv[c] * acc;
}

// residual r = f - A u on interior columns, optional sum of r^2 per block
template <typename T, bool HAS_F, bool NORM>
__global__ void __launch_bounds__(BX * BY) k_residual(View<T> v, T *r, double *partial) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    double sq = 0.0;
    if (j < v.N && k >= 1 && k <= v.K - 2) {
        const long c = (long)j * v.P + k;
        const long up = (j == 0) ? v.P : -(long)v.P;
        const long dn = (j == v.N - 1) ? -(long)v.P : v.P;
        const T *u = v.u;
        const T cW = v.cx[c - 1], cE = v.cx[c], cN = v.cz[c], cS = v.cz[c + v.P];
        const T lap = cW * u[c - 1] + cE * u[c + 1] + cN * u[c + up] + cS * u[c + dn] -
                      (((cW + cE) + cN) + cS) * u[c];
        const T res = (HAS_F ? v.f[c] : (T)0) - lap * v.inv_h2;
        r[c] = res;
        sq = (double)res * (double)res;
    }
    if (NORM) {
        sq = block_sum(sq);
        if (threadIdx.x == 0 && threadIdx.y == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = sq;
    }
}

// The level-0 residual of the mixed-precision solver, written as the FP32
// right-hand side of the correction equation, and ||r||^2 into *out.
//
// GB300 issues about one FP64 fused multiply-add per SM clock, so a
// residual in FP64 arithmetic (five per node) is bound by that pipe at a
// quarter of the bandwidth the kernel's bytes allow.  This kernel reads the
// same bytes -- u in FP64 and the moduli cx, cz and diag, stored at set-up
// as double-float pairs (d_split, 8 bytes a value like their FP64 copies)
// -- and evaluates
//   lap = cW uW + cE uE + cN uN + cS uS - diag uC
// in double-float arithmetic on the FP32 and integer pipes: each u is split
// into hi + lo on the integer pipes, each product is the exact FP32 product
// of the hi parts (the rounding error recovered by an FMA) plus the two
// cross terms, and the five hi products are summed exactly with Knuth's
// two-sum, the rounding errors and cross terms collected in FP32.  The
// error of lap is a few units of 2^-46 of sum |c u| (2^-53 for the FP64
// evaluation).  At a 1e-9 relative tolerance on a 1025^2 grid that is about
// 1 % of the tolerance's norm, spread as rounding noise uncorrelated with
// the residual, so the norm the stopping test reads moves by about 1e-4 of
// itself; the right-hand sides of the cycles, far above the tolerance, keep
// FP32's precision.  r = -lap / h^2.
//
// Layout: tiles of 30 columns x BY * RES_DF_RPT rows.  A warp covers 32
// consecutive columns of which the middle 30 are its output (the outer two
// lanes supply the west and east neighbours through shuffles), and each
// thread walks RES_DF_RPT consecutive rows of its column with its u values
// split once and kept in registers.  A grid of RES_DF_CTAS_PER_SM blocks per
// SM strides over the tiles, so that the block-wide reduction at the end
// (whose barrier idles a block's early warps) comes once per block instead
// of once per tile.  The norm sums the squares of the FP32 residual in
// FP32 throughout (residual_df_finish) -- a relative error near 1e-6 in the
// norm, which only the stopping test reads.  The last block to finish adds
// the per-block partials in a fixed order (the sum is deterministic) and
// re-arms the counter for the next launch.
static constexpr int RES_RPT = 4;          // rows per thread of the FP64 reductions (k_mr_dots)
static constexpr int RES_DF_COLS = 30;     // output columns per warp
static constexpr int RES_DF_RPT = 4;       // rows per thread
static constexpr int RES_DF_CTAS_PER_SM = 3;

__global__ void __launch_bounds__(BX * BY, RES_DF_CTAS_PER_SM)
    k_residual_df(View<double> v, const float2 *__restrict__ cx2, const float2 *__restrict__ cz2,
                  const float2 *__restrict__ dg2, float *f32, double *partial, unsigned *count, double *out,
                  Decide dc) {
    pdl_trigger();
    pdl_wait();   // launched with programmatic serialization: the previous kernel's data first
    // the graph's first check, after a prologue that found the guess
    // converged: skipped (every block reads the flag before the last block
    // of this launch could write it)
    if (dc.gate && !__ldcg(dc.gate)) return;
    constexpr int R = RES_DF_RPT;
    const int lane = threadIdx.x;
    const int N = v.N, K = v.K, P = v.P;
    const int ntx = (K - 2 + RES_DF_COLS - 1) / RES_DF_COLS, nty = (N + BY * R - 1) / (BY * R);
    const float nih2 = -(float)v.inv_h2;
    float sq = 0.f;   // squares of the FP32 residual, summed in FP32 within a warp
    for (int tile = blockIdx.x; tile < ntx * nty; tile += gridDim.x) {
        const int ty = tile / ntx, tx = tile - ty * ntx;
        const int k = tx * RES_DF_COLS + lane;                 // lanes 0 and 31: neighbours only
        const int j0 = (ty * BY + threadIdx.y) * R;
        if (j0 >= N) continue;                                  // uniform over the warp
        const bool out_col = lane >= 1 && lane <= RES_DF_COLS && k <= K - 2;
        // every load first, at clamped (always valid) indices, so that they
        // are all in flight together: u at rows j0-1 .. j0+R of this column
        // (mirrored at both ends; rows past the last are clamped, no output
        // reads them), the moduli of rows j0 .. j0+R-1 at the output column
        const int ku = min(k, K - 1), kc = max(1, min(k, K - 2));
        double uv[R + 2];
        float2 cWv[R], cEv[R], cNv[R + 1], dgv[R];
#pragma unroll
        for (int i = 0; i < R + 2; i++) {
            int j = j0 - 1 + i;
            j = j < 0 ? 1 : (j > N - 1 ? 2 * (N - 1) - j : j);
            j = max(0, min(j, N - 1));
            uv[i] = __ldg(v.u + (long)j * P + ku);
        }
#pragma unroll
        for (int i = 0; i <= R; i++) {
            const long c = (long)min(j0 + i, N) * P + kc;   // cz has N + 1 rows
            cNv[i] = __ldg(cz2 + c);
            if (i < R) {
                const long cc = (long)min(j0 + i, N - 1) * P + kc;
                cWv[i] = __ldg(cx2 + cc - 1);
                cEv[i] = __ldg(cx2 + cc);
                dgv[i] = __ldg(dg2 + cc);
            }
        }
        float uh[R + 2], ul[R + 2];
#pragma unroll
        for (int i = 0; i < R + 2; i++) {
            const float2 x = d_split(uv[i]);
            uh[i] = x.x;
            ul[i] = x.y;
        }
#pragma unroll
        for (int i = 0; i < R; i++) {
            const int j = j0 + i;
            const float wh = __shfl_up_sync(0xffffffffu, uh[i + 1], 1);
            const float wl = __shfl_up_sync(0xffffffffu, ul[i + 1], 1);
            const float eh = __shfl_down_sync(0xffffffffu, uh[i + 1], 1);
            const float el = __shfl_down_sync(0xffffffffu, ul[i + 1], 1);
            if (out_col && j < N) {
                float s, lo;
                df_first(cWv[i].x, cWv[i].y, wh, wl, s, lo);
                df_acc(cEv[i].x, cEv[i].y, eh, el, s, lo);
                df_acc(cNv[i].x, cNv[i].y, uh[i], ul[i], s, lo);
                df_acc(cNv[i + 1].x, cNv[i + 1].y, uh[i + 2], ul[i + 2], s, lo);
                df_acc(-dgv[i].x, -dgv[i].y, uh[i + 1], ul[i + 1], s, lo);
                const float r = __fadd_rn(s, lo) * nih2;
                f32[(long)j * P + k] = r;
                sq = fmaf(r, r, sq);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    // The reductions from here on run in binary32, as the squares within
    // each warp did: the norm is good to about 1e-6 of itself either way
    // (only the stopping test reads it), and a chain of dependent FP64
    // additions costs about 130 clocks an addition on GB300's FP64 pipe
    // against 4 in binary32.  The block sums go to `partial` as floats.
    __shared__ float wsum[BX * BY / 32];
    __shared__ bool last;
    float *pf = reinterpret_cast<float *>(partial);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const unsigned nblk = gridDim.x;   // a one-dimensional grid
    // mode 1 with the relative tolerance: ||r0||^2 of the zero-interior
    // guess (as k_r0: only the columns next to the Dirichlet data see a
    // residual), its rows dealt round-robin to the blocks, each row in FP64
    // and the sums as double-float pairs (||r0|| sets the threshold and is
    // reported, so it keeps FP64's precision), each block's first warp
    // summing its few rows into pf[nblk + 2 block ..]
    const bool r0_rows = dc.mode == 1 && dc.rel;
    float2 r0b = make_float2(0.f, 0.f);
    if (r0_rows && tid < 32) {
        double acc = 0.0;
        for (int j = tid * (int)nblk + (int)blockIdx.x; j < v.N; j += 32 * (int)nblk) {
            const long row = (long)j * v.P;
            if (v.K - 2 == 1) {
                const double r = -(v.cx[row] * v.u[row] + v.cx[row + 1] * v.u[row + 2]) * v.inv_h2;
                acc += r * r;
            } else if (v.K - 2 > 1) {
                const double r1 = -v.cx[row] * v.u[row] * v.inv_h2;
                const double r2 = -v.cx[row + v.K - 2] * v.u[row + v.K - 1] * v.inv_h2;
                acc += r1 * r1 + r2 * r2;
            }
        }
        r0b = df_of(acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            r0b = df_add(r0b, make_float2(__shfl_xor_sync(0xffffffffu, r0b.x, o), __shfl_xor_sync(0xffffffffu, r0b.y, o)));
    }
    if ((tid & 31) == 0) wsum[tid >> 5] = sq;
    __syncthreads();
    if (tid == 0) {
        float b = 0.f;
        for (int w = 0; w < BX * BY / 32; w++) b += wsum[w];
        pf[blockIdx.x] = b;
        if (r0_rows) {
            pf[nblk + 2 * blockIdx.x] = r0b.x;
            pf[nblk + 2 * blockIdx.x + 1] = r0b.y;
        }
        __threadfence();
        last = atomicAdd(count, 1u) == nblk - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the last block: the block sums in a fixed order (deterministic)
    float t = 0.f;
    for (unsigned i = tid; i < nblk; i += blockDim.x * blockDim.y) t += __ldcg(pf + i);
    t = block_sum_f(t);
    float2 r0 = make_float2(0.f, 0.f);
    if (r0_rows) {
        for (unsigned i = tid; i < nblk; i += blockDim.x * blockDim.y)
            r0 = df_add(r0, make_float2(__ldcg(pf + nblk + 2 * i), __ldcg(pf + nblk + 2 * i + 1)));
        r0 = block_sum_df(r0);
    }
    if (tid != 0) return;
    *out = f2d_exact(t);
    *count = 0;
    const double delta = f2d_exact(sqrtf(t));
    if (dc.mode == 1) {
        const double r0sq = f2d_exact(r0.x) + f2d_exact(r0.y);
        if (dc.rel) out[1] = r0sq;
        const int go = solve_begin_dev(delta, sqrt_refined(r0sq), dc.st, dc.rel, dc.tol, dc.n_kernels, dc.phase,
                                       dc.net_ratio, dc.n_kernels_gated);
        if (dc.in_graph) {
            cudaGraphSetConditional(dc.h, go ? 1u : 0u);
            if (dc.phase == 1) cudaGraphSetConditional(dc.h_net, dc.st->net ? 1u : 0u);
        }
    } else if (dc.mode == 2) {
        const int go = solve_check_dev(delta, dc.st, dc.max_cycles, dc.n_kernels, dc.smooth_ratio, dc.n_kernels_smooth);
        if (dc.in_graph) {
            cudaGraphSetConditional(dc.h, go ? 1u : 0u);
            if (dc.smooth_ratio > 1.0) cudaGraphSetConditional(dc.h_smooth, dc.st->smooth ? 1u : 0u);
        }
    }
}

// the double-float moduli of level 0 (d_split of cx, cz and diag)
__global__ void k_split_moduli(int N, int P, const double *cx, const double *cz, const double *diag, float2 *cx2,
                               float2 *cz2, float2 *dg2) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long n = (long)N * P;
    if (i < n) {
        cx2[i] = d_split(cx[i]);
        dg2[i] = d_split(diag[i]);
    }
    if (i < n + P) cz2[i] = d_split(cz[i]);
}

// residual norm^2 of the zero-interior guess: only the columns next to the
// Dirichlet data see a non-zero residual (f = 0 on level 0).  One block: each
// thread sums its rows, the block reduces in a fixed order into *out.
template <typename T>
__global__ void __launch_bounds__(1024) k_r0(View<T> v, double *out) {
    double sq = 0.0;
    for (int j = threadIdx.x; j < v.N; j += blockDim.x) {
        const long row = (long)j * v.P;
        const int K = v.K;
        if (K - 2 == 1) {
            const double r = -((double)v.cx[row] * v.u[row] + (double)v.cx[row + 1] * v.u[row + 2]) *
                             (double)v.inv_h2;
            sq += r * r;
        } else if (K - 2 > 1) {
            const double r1 = -(double)v.cx[row] * (double)v.u[row] * (double)v.inv_h2;
            const double r2 = -(double)v.cx[row + K - 2] * (double)v.u[row + K - 1] * (double)v.inv_h2;
            sq += r1 * r1 + r2 * r2;
        }
    }
    sq = block_sum(sq);
    if (threadIdx.x == 0) *out = sq;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <typename T>
static T *dalloc(size_t n, int *rc) {
    T *p = nullptr;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
        *rc = QD_ERR_NOMEM;
        return nullptr;
    }
    cudaMemset(p, 0, n * sizeof(T));
    return p;
}

int mg_alloc(qd_solver *s, const double *mu_equi_host, const double *jrow_host) {
    const int nl = s->opt.n_levels;
    if (nl < 1 || nl > QD_MAXLEV) {
        set_error("n_levels %d out of range 1..%d", nl, QD_MAXLEV);
        return QD_ERR_ARG;
    }
    int N = s->nk, K = s->ni;
    double h = s->dh;
    for (int l = 0; l < nl; l++) {
        if (l > 0) {
            if ((N - 1) % 2 || (K - 1) % 2) {
                set_error("grid %dx%d not coarsenable to %d levels", s->nk, s->ni, nl);
                return QD_ERR_ARG;
            }
            N = (N - 1) / 2 + 1;
            K = (K - 1) / 2 + 1;
            h *= 2;
        }
        if (N < 3 || K < 3) {
            set_error("level %d has %dx%d nodes (< 3)", l, N, K);
            return QD_ERR_ARG;
        }
        s->dims[l].N = N; s->dims[l].K = K; s->dims[l].P = cdiv(K, 32) * 32;
        s->dims[l].h2 = h * h;
        s->dims[l].inv_h2 = 1.0 / (h * h);
    }
    s->nlev = nl;
    {
        int dev = 0;
        QD_CUDA(cudaGetDevice(&dev));
        QD_CUDA(cudaDeviceGetAttribute(&s->n_sm, cudaDevAttrMultiProcessorCount, dev));
    }
    int rc = QD_OK;
    for (int l = 0; l < nl; l++) {
        const size_t n = (size_t)s->dims[l].N * s->dims[l].P;
        const size_t nf = (size_t)(s->dims[l].N + 1) * s->dims[l].P;
        s->L64[l].u = dalloc<double>(n, &rc);
        s->L64[l].r = dalloc<double>(n, &rc);
        s->L64[l].f = l > 0 ? dalloc<double>(n, &rc) : nullptr;
        s->L64[l].cx = dalloc<double>(n, &rc);
        s->L64[l].cz = dalloc<double>(nf, &rc);
        s->L64[l].dinv = dalloc<double>(n, &rc);
        s->L64[l].diag = l == 0 ? dalloc<double>(n, &rc) : nullptr;
        s->L32[l].u = dalloc<float>(n, &rc);
        s->L32[l].r = dalloc<float>(n, &rc);
        s->L32[l].f = dalloc<float>(n, &rc);
        s->L32[l].cx = dalloc<float>(n, &rc);
        s->L32[l].cz = dalloc<float>(nf, &rc);
        s->L32[l].dinv = dalloc<float>(n, &rc);
        if (rc != QD_OK) {
            set_error("device allocation failed on level %d", l);
            return rc;
        }
    }
    if (s->opt.precision == QD_PREC_MIXED) {
        const size_t n = (size_t)s->dims[0].N * s->dims[0].P;
        s->res_cx = dalloc<float2>(n, &rc);
        s->res_cz = dalloc<float2>(n + s->dims[0].P, &rc);
        s->res_dg = dalloc<float2>(n, &rc);
        if (rc != QD_OK) {
            set_error("device allocation failed (level-0 double-float moduli)");
            return rc;
        }
    }
    s->n_partial = cdiv(s->dims[0].K, BX) * cdiv(s->dims[0].N, BY) + 64;
    s->d_partial = dalloc<double>(s->n_partial, &rc);
    s->d_count = dalloc<unsigned>(1, &rc);
    if (rc != QD_OK) return rc;
    QD_CUDA(cudaMemsetAsync(s->d_count, 0, sizeof(unsigned), s->stream));

    // coefficients from mu_equi
    const size_t nmu = (size_t)(2 * s->nx - 1) * (2 * s->nz - 1);
    double *d_mu = dalloc<double>(nmu, &rc);
    if (rc != QD_OK) return rc;
    QD_CUDA(cudaMemcpyAsync(d_mu, mu_equi_host, nmu * sizeof(double), cudaMemcpyHostToDevice,
                            s->stream));
    double *d_j = nullptr;
    if (jrow_host) {
        const size_t nj = 2 * (size_t)s->nz - 1;
        d_j = dalloc<double>(nj, &rc);
        if (rc != QD_OK) return rc;
        QD_CUDA(cudaMemcpyAsync(d_j, jrow_host, nj * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    }
    const long W = 2L * s->nx - 1;
    for (int l = 0; l < nl; l++) {
        const LevelDims &d = s->dims[l];
        dim3 blk(BX, BY), grd(cdiv(d.K, BX), cdiv(d.N + 1, BY));
        k_build_faces<<<grd, blk, 0, s->stream>>>(d_mu, d_j, W, l, 1 << l, d.N, d.K, d.P, s->L64[l].cx,
                                                  s->L64[l].cz);
        QD_LAUNCH_CHECK(s);
        k_build_dinv<<<grd, blk, 0, s->stream>>>(d.N, d.K, d.P, s->L64[l].cx, s->L64[l].cz,
                                                 s->L64[l].dinv, s->L32[l].cx, s->L32[l].cz,
                                                 s->L32[l].dinv, s->L64[l].diag);
        QD_LAUNCH_CHECK(s);
    }
    if (s->res_cx) {
        const LevelDims &d = s->dims[0];
        const long n = (long)(d.N + 1) * d.P;
        k_split_moduli<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(d.N, d.P, s->L64[0].cx, s->L64[0].cz,
                                                                           s->L64[0].diag, s->res_cx, s->res_cz,
                                                                           s->res_dg);
        QD_LAUNCH_CHECK(s);
    }
    QD_CUDA(cudaStreamSynchronize(s->stream));
    cudaFree(d_mu);
    cudaFree(d_j);
    QD_TRY(build_coarse_inverse(s));
    return tail_image_build(s);
}

// Dense inverse of the coarsest level's operator, for the exact coarse solve
// (qd_mg_options.coarse_solve).  Row (j,k) of A holds the equation the
// smoother relaxes, (sum_nb c_nb e_nb - diag e) / h^2 = f, over the interior
// columns with the mirrored rows and zero Dirichlet columns; Gauss-Jordan
// with partial pivoting in FP64 on the host, once.
int build_coarse_inverse(qd_solver *s) {
    const int l = s->nlev - 1;
    const LevelDims &d = s->dims[l];
    const int N = d.N, K = d.K, P = d.P, n = N * (K - 2);
    s->n_cint = 0;
    if (s->nlev < 2 || n > 1024) return QD_OK;   // coarse_solve then rejected by the solve
    std::vector<double> cx((size_t)N * P), cz((size_t)(N + 1) * P);
    QD_CUDA(cudaMemcpy(cx.data(), s->L64[l].cx, cx.size() * sizeof(double), cudaMemcpyDeviceToHost));
    QD_CUDA(cudaMemcpy(cz.data(), s->L64[l].cz, cz.size() * sizeof(double), cudaMemcpyDeviceToHost));
    auto id = [K](int j, int k) { return j * (K - 2) + (k - 1); };
    const double ih2 = 1.0 / d.h2;
    std::vector<double> A((size_t)n * n, 0.0), B((size_t)n * n, 0.0);
    for (int j = 0; j < N; j++)
        for (int k = 1; k <= K - 2; k++) {
            const long c = (long)j * P + k;
            const double cW = cx[c - 1], cE = cx[c], cN = cz[c], cS = cz[c + P];
            const long row = (long)id(j, k) * n;
            A[row + id(j, k)] -= (((cW + cE) + cN) + cS) * ih2;
            if (k - 1 >= 1) A[row + id(j, k - 1)] += cW * ih2;
            if (k + 1 <= K - 2) A[row + id(j, k + 1)] += cE * ih2;
            const int jn = (j == 0) ? 1 : j - 1, js = (j == N - 1) ? N - 2 : j + 1;
            A[row + id(jn, k)] += cN * ih2;
            A[row + id(js, k)] += cS * ih2;
        }
    for (int i = 0; i < n; i++) B[(long)i * n + i] = 1.0;
    for (int c = 0; c < n; c++) {
        int p = c;
        for (int r = c + 1; r < n; r++)
            if (fabs(A[(long)r * n + c]) > fabs(A[(long)p * n + c])) p = r;
        if (A[(long)p * n + c] == 0.0) {
            set_error("coarsest-level operator is singular");
            return QD_ERR_ARG;
        }
        if (p != c)
            for (int m = 0; m < n; m++) {
                std::swap(A[(long)p * n + m], A[(long)c * n + m]);
                std::swap(B[(long)p * n + m], B[(long)c * n + m]);
            }
        const double inv = 1.0 / A[(long)c * n + c];
        for (int m = 0; m < n; m++) {
            A[(long)c * n + m] *= inv;
            B[(long)c * n + m] *= inv;
        }
        for (int r = 0; r < n; r++) {
            if (r == c) continue;
            const double f = A[(long)r * n + c];
            if (f == 0.0) continue;
            for (int m = 0; m < n; m++) {
                A[(long)r * n + m] -= f * A[(long)c * n + m];
                B[(long)r * n + m] -= f * B[(long)c * n + m];
            }
        }
    }
    std::vector<float> B32(B.size());
    for (size_t i = 0; i < B.size(); i++) B32[i] = (float)B[i];
    QD_CUDA(cudaMalloc(&s->d_ainv64, B.size() * sizeof(double)));
    QD_CUDA(cudaMalloc(&s->d_ainv32, B.size() * sizeof(float)));
    QD_CUDA(cudaMemcpy(s->d_ainv64, B.data(), B.size() * sizeof(double), cudaMemcpyHostToDevice));
    QD_CUDA(cudaMemcpy(s->d_ainv32, B32.data(), B32.size() * sizeof(float), cudaMemcpyHostToDevice));
    s->n_cint = n;
    return QD_OK;
}

void mg_free(qd_solver *s) {
    for (int l = 0; l < QD_MAXLEV; l++) {
        cudaFree(s->L64[l].u); cudaFree(s->L64[l].r); cudaFree(s->L64[l].f);
        cudaFree(s->L64[l].cx); cudaFree(s->L64[l].cz); cudaFree(s->L64[l].dinv);
        cudaFree(s->L64[l].diag);
        cudaFree(s->L32[l].u); cudaFree(s->L32[l].r); cudaFree(s->L32[l].f);
        cudaFree(s->L32[l].cx); cudaFree(s->L32[l].cz); cudaFree(s->L32[l].dinv);
        s->L64[l] = Level<double>();
        s->L32[l] = Level<float>();
    }
    cudaFree(s->res_cx);
    cudaFree(s->res_cz);
    cudaFree(s->res_dg);
    s->res_cx = s->res_cz = s->res_dg = nullptr;
    cudaFree(s->d_partial);
    cudaFree(s->d_count);
    s->d_count = nullptr;
    cudaFree(s->d_ainv64);
    cudaFree(s->d_ainv32);
    tma_cache_free(s);
    tail_image_free(s);
    s->d_ainv64 = nullptr;
    s->d_ainv32 = nullptr;
    s->d_partial = nullptr;
}

template <typename T>
static int smooth_t(qd_solver *s, Level<T> *Ls, int l, int nsweeps) {
    View<T> v = make_view(s, Ls, l);
    dim3 blk(BX, BY), grd(cdiv((v.K - 1) / 2 + 1, BX), cdiv(v.N, BY));
    for (int it = 0; it < nsweeps; it++) {
        for (int color = 0; color < 2; color++) {
            if (v.f)
                k_rb<T, true><<<grd, blk, 0, s->stream>>>(v, color);
            else
                k_rb<T, false><<<grd, blk, 0, s->stream>>>(v, color);
            QD_LAUNCH_CHECK(s);
        }
    }
    return QD_OK;
}

// The energy-optimal step along a correction of the guess.  With u0 the
// guess, d = u - u0 the correction already added to u (zero on the boundary
// columns), A x = lap(x) / h^2 the level-0 operator of the residual kernels
// (negative definite) and r0 = f - A u0 = A e (e: the guess's error),
// alpha = (d . r0) / (d . A d) minimises the error's energy norm
// (e - alpha d)^T (-A) (e - alpha d) -- the Galerkin step of a one-vector
// subspace -- so the corrected guess u0 + alpha d never has a larger error
// in that norm than u0 (alpha = 1 for an exact correction, 0 when d . A d
// is not negative).  The residual norm, which weights the correction's
// high-frequency content, is not the measure: a prediction that is right in
// the smooth components and noisy in the rough ones still saves V-cycles.
// k_mr_dots: both sums per block, the last block adds the partials in a
// fixed order and writes alpha; k_mr_update: u = u0 + alpha d.
template <bool HAS_F>
__global__ void __launch_bounds__(BX * BY)
    k_mr_dots(View<double> v, const double *__restrict__ diag, const double *__restrict__ u0, double *partial,
              unsigned *count, double *alpha) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j0 = blockIdx.y * (BY * RES_RPT) + threadIdx.y;
    double ra = 0.0, aa = 0.0;
    if (k >= 1 && k <= v.K - 2) {
        const double *__restrict__ u = v.u;
#pragma unroll
        for (int i = 0; i < RES_RPT; i++) {
            const int j = j0 + i * BY;
            if (j < v.N) {
                const long c = (long)j * v.P + k;
                const long up = (j == 0) ? v.P : -(long)v.P;
                const long dn = (j == v.N - 1) ? -(long)v.P : v.P;
                const double a0 = u0[c - 1], a1 = u0[c + 1], a2 = u0[c + up], a3 = u0[c + dn], a4 = u0[c];
                const double lap0 = v.cx[c - 1] * a0 + v.cx[c] * a1 + v.cz[c] * a2 + v.cz[c + v.P] * a3 - diag[c] * a4;
                const double lapd = v.cx[c - 1] * (u[c - 1] - a0) + v.cx[c] * (u[c + 1] - a1) +
                                    v.cz[c] * (u[c + up] - a2) + v.cz[c + v.P] * (u[c + dn] - a3) -
                                    diag[c] * (u[c] - a4);
                const double r0 = HAS_F ? v.f[c] - lap0 * v.inv_h2 : -lap0 * v.inv_h2;
                const double dc = u[c] - a4;
                ra = fma(dc, r0, ra);                 // d . r0
                aa = fma(dc, lapd * v.inv_h2, aa);    // d . A d (< 0)
            }
        }
    }
    ra = block_sum(ra);
    aa = block_sum(aa);
    __shared__ bool last;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const unsigned nblk = gridDim.x * gridDim.y;
    if (tid == 0) {
        const unsigned b = blockIdx.y * gridDim.x + blockIdx.x;
        partial[2 * b] = ra;
        partial[2 * b + 1] = aa;
        __threadfence();
        last = atomicAdd(count, 1u) == nblk - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    ra = 0.0;
    aa = 0.0;
    for (unsigned i = tid; i < nblk; i += blockDim.x * blockDim.y) {
        ra += __ldcg(partial + 2 * i);
        aa += __ldcg(partial + 2 * i + 1);
    }
    ra = block_sum(ra);
    aa = block_sum(aa);
    if (tid == 0) {
        const double al = ra / aa;
        *alpha = (aa < 0.0 && isfinite(al)) ? al : 0.0;
        *count = 0;
    }
}

__global__ void k_mr_update(double *u, const double *u0, int N, int K, int P, const double *alpha) {
    const int j = blockIdx.y, k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j >= N || k > K - 2) return;
    const long c = (long)j * P + k;
    const double a = *alpha;
    u[c] = a == 0.0 ? u0[c] : u0[c] + a * (u[c] - u0[c]);   // alpha 0 also drops a non-finite correction
}

int mr_step(qd_solver *s, const double *u0) {
    View<double> v = make_view(s, s->L64, 0);
    dim3 blk(BX, BY), grd(cdiv(v.K, BX), cdiv(v.N, BY * RES_RPT));
    if (2 * (long)grd.x * grd.y > s->n_partial) {
        set_error("minimal-residual step: %u blocks exceed the partial buffer", grd.x * grd.y);
        return QD_ERR_ARG;
    }
    double *alpha = s->d_scal + 3;
    if (v.f)
        k_mr_dots<true><<<grd, blk, 0, s->stream>>>(v, s->L64[0].diag, u0, s->d_partial, s->d_count, alpha);
    else
        k_mr_dots<false><<<grd, blk, 0, s->stream>>>(v, s->L64[0].diag, u0, s->d_partial, s->d_count, alpha);
    QD_LAUNCH_CHECK(s);
    k_mr_update<<<dim3(cdiv(v.K, 256), v.N), 256, 0, s->stream>>>(v.u, u0, v.N, v.K, v.P, alpha);
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

// the mixed solver's level-0 residual (k_residual_df) into the FP32
// right-hand side, ||r||^2 into d_scal[slot] and the decision dc
static int residual_df(qd_solver *s, const Decide &dc, int slot, bool pdl) {
    if (!s->res_cx) {
        set_error("level-0 residual: the double-float moduli exist only in mixed precision");
        return QD_ERR_STATE;
    }
    View<double> v = make_view(s, s->L64, 0);
    const int tiles = cdiv(v.K - 2, RES_DF_COLS) * cdiv(v.N, BY * RES_DF_RPT);
    dim3 blk(BX, BY), grd(std::min(tiles, RES_DF_CTAS_PER_SM * s->n_sm));
    if (2 * (long)grd.x > s->n_partial) {   // the squares' and ||r0||'s block sums
        set_error("level-0 residual: %u blocks exceed the partial buffer", grd.x);
        return QD_ERR_ARG;
    }
    QD_CUDA(launch_pdl(pdl, k_residual_df, grd, blk, 0, s->stream, v, (const float2 *)s->res_cx,
                       (const float2 *)s->res_cz, (const float2 *)s->res_dg, s->L32[0].f, s->d_partial, s->d_count,
                       s->d_scal + slot, dc));
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

// the mixed solver's level-0 residual with a decision fused into its last
// block (norm into d_scal[0], ||r0||^2 into d_scal[1] for mode 1)
int level0_norm_decide(qd_solver *s, const Decide &dc) {
    QD_TRY(residual_df(s, dc, 0, true));
    return QD_OK;
}

// ||r||^2 of level 0 into d_scal[slot]: in FP64 (to32 = 0), or the mixed
// solver's residual, which also writes the FP32 correction right-hand side
int level0_norm(qd_solver *s, int to32, int slot) {
    View<double> v = make_view(s, s->L64, 0);
    if (to32) {
        QD_TRY(residual_df(s, Decide{}, slot, false));
        return QD_OK;
    }
    dim3 blk(BX, BY), grd(cdiv(v.K, BX), cdiv(v.N, BY));
    const int nb = grd.x * grd.y;
    k_residual<double, false, true><<<grd, blk, 0, s->stream>>>(v, v.r, s->d_partial);
    QD_LAUNCH_CHECK(s);
    k_final_sum<<<1, 1024, 0, s->stream>>>(s->d_partial, nb, s->d_scal + slot);
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

int r0_norm(qd_solver *s, int slot) {
    View<double> v = make_view(s, s->L64, 0);
    k_r0<double><<<1, 1024, 0, s->stream>>>(v, s->d_scal + slot);
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

static int read_scalars(qd_solver *s, int n) {
    QD_CUDA(cudaMemcpyAsync(s->h_scal, s->d_scal, n * sizeof(double), cudaMemcpyDeviceToHost,
                            s->stream));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    return QD_OK;
}

// nsweeps red+black sweeps of the level-`level` field of the hierarchy the
// solver's precision runs its cycles in (FP64 u, or the FP32 correction)
int mg_smooth(qd_solver *s, int level, int nsweeps) {
    if (s->opt.precision == QD_PREC_MIXED)
        QD_TRY(smooth_t<float>(s, s->L32, level, nsweeps));
    else
        QD_TRY(smooth_t<double>(s, s->L64, level, nsweeps));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    return QD_OK;
}

int mg_vcycle(qd_solver *s) {
    int nb = 0;
    QD_TRY(vcycle64_norm(s, &nb));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    return QD_OK;
}

int mg_residual_norm(qd_solver *s, double *rnorm) {
    QD_TRY(level0_norm(s, 0, 0));
    QD_TRY(read_scalars(s, 1));
    *rnorm = sqrt(s->h_scal[0]);
    return QD_OK;
}

__global__ void k_d2f(const double *in, float *out, int n, float *lo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (lo) {
        const float2 x = d_split(in[i]);
        out[i] = x.x;
        lo[i] = x.y;
    } else {
        out[i] = d2f_rne(in[i]);
    }
}

// d2f_rne (lo null) or d_split over a host array (a device round trip), for
// their tests
int convert_f64_f32(const double *in, float *out, int n, float *lo) {
    double *din = nullptr;
    float *dout = nullptr, *dlo = nullptr;
    int rc = QD_OK;
    if (cudaMalloc(&din, sizeof(double) * (size_t)n) != cudaSuccess ||
        cudaMalloc(&dout, sizeof(float) * (size_t)n) != cudaSuccess ||
        (lo && cudaMalloc(&dlo, sizeof(float) * (size_t)n) != cudaSuccess) ||
        cudaMemcpy(din, in, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess) {
        rc = QD_ERR_CUDA;
    } else {
        k_d2f<<<cdiv(n, 256), 256>>>(din, dout, n, dlo);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(out, dout, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess ||
            (lo && cudaMemcpy(lo, dlo, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess))
            rc = QD_ERR_CUDA;
    }
    if (rc != QD_OK) {
        (void)cudaGetLastError();
        set_error("convert_f64_f32: CUDA failure");
    }
    cudaFree(din);
    cudaFree(dout);
    cudaFree(dlo);
    return rc;
}

}  // namespace qd
