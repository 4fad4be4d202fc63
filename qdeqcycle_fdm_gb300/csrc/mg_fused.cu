// mg_fused.cu -- the V-cycle as shared-memory tile kernels.
//
// Red-black Gauss-Seidel sweeps are temporally blocked: a CTA stages a tile
// of u, f and the face moduli with a halo as wide as the number of
// half-sweeps S, runs all S half-sweeps in shared memory (each half-sweep
// invalidates one more ring of the halo) and writes back only its core.
// Each update is the same expression as the one-colour kernel in mg.cu, so
// the result equals S global half-sweeps bit for bit.
//
// Per fine level l of a V-cycle:
//   k_down<l>: [zero guess] -> S_pre half-sweeps -> residual -> full-weighting
//              restriction to level l+1's right-hand side (one launch)
//   k_up<l>:   bilinear prolongation of level l+1's correction -> S_post
//              half-sweeps [-> residual norm on level 0 | -> u64 += e on
//              level 0 of the mixed-precision cycle] (one launch)
// and every level of at most TAIL_N rows runs inside one single-CTA kernel
// (k_tail) that performs that part of the V-cycle with block barriers.
//
// Coarse-level corrections always start from zero, so the coarse k_down
// never reads u (the reference zeroes e2 in restriction_kernel and then
// reads it back).
#include <algorithm>

#include "qdeq_internal.cuh"

namespace qd {

static constexpr int NT = 512;        // threads of the tile kernels
static constexpr int NT_TAIL = 1024;  // threads of the coarse-tail kernel
static constexpr int TAIL_N = 65;     // levels with at most this many rows run in the tail
static constexpr int SMAX = 8;        // half-sweeps per tile pass

template <typename T>
struct LvArgs {
    T *u;
    const T *f;
    const T *cx, *cz, *dinv;
    T *r;
    int N, K, P;
    T h2, inv_h2;
};

template <typename T>
static LvArgs<T> lv(const qd_solver *s, const Level<T> *Ls, int l) {
    LvArgs<T> a;
    a.u = Ls[l].u; a.f = Ls[l].f; a.cx = Ls[l].cx; a.cz = Ls[l].cz; a.dinv = Ls[l].dinv;
    a.r = Ls[l].r;
    a.N = s->dims[l].N; a.K = s->dims[l].K; a.P = s->dims[l].P;
    a.h2 = (T)s->dims[l].h2; a.inv_h2 = (T)s->dims[l].inv_h2;
    return a;
}

// ---------------------------------------------------------------------------
// shared-memory tile
// ---------------------------------------------------------------------------
template <typename T>
struct STile {
    T *u, *f, *cx, *cz, *dv;
    int jL0, kL0, LR, LC;
};

template <typename T>
__device__ __forceinline__ STile<T> carve(unsigned char *raw, int jL0, int kL0, int LR, int LC, bool has_f) {
    STile<T> t;
    t.jL0 = jL0; t.kL0 = kL0; t.LR = LR; t.LC = LC;
    const int n = LR * LC;
    T *p = reinterpret_cast<T *>(raw);
    t.u = p; p += n;
    t.cx = p; p += n;
    t.dv = p; p += n;
    t.cz = p; p += n + LC;
    t.f = has_f ? p : nullptr;
    return t;
}

static size_t tile_bytes(size_t esz, int LR, int LC, bool has_f) {
    return esz * ((size_t)LR * LC * (has_f ? 5 : 4) + LC);
}

template <typename T>
__device__ void tile_load(const LvArgs<T> &g, STile<T> &t, bool zero_u) {
    const int n = t.LR * t.LC;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int r = i / t.LC, c = i - r * t.LC;
        const long gi = (long)(t.jL0 + r) * g.P + t.kL0 + c;
        t.u[i] = zero_u ? (T)0 : g.u[gi];
        t.cx[i] = g.cx[gi];
        t.dv[i] = g.dinv[gi];
        if (t.f) t.f[i] = g.f[gi];
    }
    const int nz = (t.LR + 1) * t.LC;
    for (int i = threadIdx.x; i < nz; i += blockDim.x) {
        const int r = i / t.LC, c = i - r * t.LC;
        t.cz[i] = g.cz[(long)(t.jL0 + r) * g.P + t.kL0 + c];
    }
}

// one colour over the tile; nodes whose neighbours are not in the tile are
// skipped (they lie in the part of the halo that is already stale)
template <typename T>
__device__ void tile_halfsweep(const LvArgs<T> &g, const STile<T> &t, int color) {
    const int HC = (t.LC + 1) >> 1;
    const int n = t.LR * HC;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int r = i / HC, m = i - r * HC;
        const int j = t.jL0 + r;
        const int c = 2 * m + ((color + j + t.kL0) & 1);
        if (c < 1 || c > t.LC - 2) continue;
        const int k = t.kL0 + c;
        if (k < 1 || k > g.K - 2) continue;
        const int rn = (j == 0) ? r + 1 : r - 1;
        const int rs = (j == g.N - 1) ? r - 1 : r + 1;
        if (rn < 0 || rn >= t.LR || rs < 0 || rs >= t.LR) continue;
        const int idx = r * t.LC + c;
        T acc = t.cx[idx - 1] * t.u[idx - 1] + t.cx[idx] * t.u[idx + 1] + t.cz[idx] * t.u[rn * t.LC + c] +
                t.cz[idx + t.LC] * t.u[rs * t.LC + c];
        if (t.f) acc -= g.h2 * t.f[idx];
        t.u[idx] = t.dv[idx] * acc;
    }
}

// residual at local (r, c) of global row j (interior column, neighbours in tile)
template <typename T>
__device__ __forceinline__ T tile_residual(const LvArgs<T> &g, const STile<T> &t, int r, int c, int j) {
    const int rn = (j == 0) ? r + 1 : r - 1;
    const int rs = (j == g.N - 1) ? r - 1 : r + 1;
    const int idx = r * t.LC + c;
    const T cW = t.cx[idx - 1], cE = t.cx[idx], cN = t.cz[idx], cS = t.cz[idx + t.LC];
    const T lap = cW * t.u[idx - 1] + cE * t.u[idx + 1] + cN * t.u[rn * t.LC + c] + cS * t.u[rs * t.LC + c] -
                  (((cW + cE) + cN) + cS) * t.u[idx];
    return (t.f ? t.f[idx] : (T)0) - lap * g.inv_h2;
}

__device__ static double block_sum_1d(double v) {
    __shared__ double sh[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = (threadIdx.x < (blockDim.x + 31) / 32) ? sh[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;
}

// ---------------------------------------------------------------------------
// k_down: pre-smoothing + residual + restriction, one coarse tile per CTA
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(NT)
    k_down(LvArgs<T> g, LvArgs<T> c, int CH, int CW, int ntj, int ntk, int S, int zero_u) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tj = blockIdx.y, tk = blockIdx.x;
    const int cj0 = tj * CH, cj1 = (tj == ntj - 1) ? c.N : cj0 + CH;
    const int ck0 = tk * CW, ck1 = (tk == ntk - 1) ? c.K : ck0 + CW;
    const int jL0 = max(0, 2 * cj0 - 2 - S), jL1 = min(g.N, 2 * cj1 + S + 1);
    const int kL0 = max(0, 2 * ck0 - 2 - S), kL1 = min(g.K, 2 * ck1 + S + 1);
    STile<T> t = carve<T>(smem, jL0, kL0, jL1 - jL0, kL1 - kL0, g.f != nullptr);
    tile_load(g, t, zero_u != 0);
    __syncthreads();
    for (int s = 0; s < S; s++) {
        tile_halfsweep(g, t, s & 1);
        __syncthreads();
    }
    // residual on fine rows 2cj0-1 .. 2cj1-1, columns 2ck0-1 .. 2ck1-1, into
    // dv (1/diag is no longer needed and the residual does not read it)
    {
        const int ja = max(0, 2 * cj0 - 1), jb = min(g.N - 1, 2 * cj1 - 1);
        const int ka = max(1, 2 * ck0 - 1), kb = min(g.K - 2, 2 * ck1 - 1);
        const int W = kb - ka + 1, n = (jb - ja + 1) * W;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int rr = i / W, cc = i - rr * W;
            const int j = ja + rr, k = ka + cc;
            t.dv[(j - jL0) * t.LC + (k - kL0)] = tile_residual(g, t, j - jL0, k - kL0, j);
        }
    }
    __syncthreads();
    // restriction onto owned coarse nodes (restriction_kernel, :953-1015)
    {
        const int ka = max(1, ck0), kb = min(c.K - 2, ck1 - 1);
        const int W = kb - ka + 1, n = (cj1 - cj0) * W;
        for (int i = threadIdx.x; i < n && W > 0; i += blockDim.x) {
            const int rr = i / W, cc = i - rr * W;
            const int j = cj0 + rr, k = ka + cc;
            const int rn = (j == 0) ? 2 * j + 1 : 2 * j - 1;
            const int rs = (j == c.N - 1) ? 2 * j - 1 : 2 * j + 1;
            const T *c0 = t.dv + (2 * j - jL0) * t.LC + (2 * k - kL0);
            const T *cn = t.dv + (rn - jL0) * t.LC + (2 * k - kL0);
            const T *cs = t.dv + (rs - jL0) * t.LC + (2 * k - kL0);
            const T val = (T)0.06250 * ((T)4.0 * c0[0] + (T)2.0 * c0[-1] + (T)2.0 * c0[1] +
                                        (T)2.0 * cn[0] + (T)2.0 * cs[0] + cn[-1] + cn[1] + cs[-1] + cs[1]);
            ((T *)c.f)[(long)j * c.P + k] = val;
        }
    }
    // smoothed fine u on the owned region
    {
        const int ja = 2 * cj0, jb = min(g.N, 2 * cj1);
        const int ka = max(1, 2 * ck0), kb = min(g.K - 1, 2 * ck1);
        const int W = kb - ka, n = (jb - ja) * W;
        for (int i = threadIdx.x; i < n && W > 0; i += blockDim.x) {
            const int rr = i / W, cc = i - rr * W;
            const int j = ja + rr, k = ka + cc;
            g.u[(long)j * g.P + k] = t.u[(j - jL0) * t.LC + (k - kL0)];
        }
    }
}

// ---------------------------------------------------------------------------
// k_up: prolongation + post-smoothing, one fine tile per CTA.
// MODE 0: write u back; 1: also residual norm partials (needs a one-wider
// halo); 2: add the smoothed correction to the FP64 field u64 instead.
// prolong = 0 turns it into a plain S-half-sweep tile smoother.
// ---------------------------------------------------------------------------
template <typename T, int MODE>
__global__ void __launch_bounds__(NT)
    k_up(LvArgs<T> g, LvArgs<T> c, int TH, int TW, int ntj, int ntk, int S, int prolong,
         int surface, int zero_u, double *partial, double *u64, int P64) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tj = blockIdx.y, tk = blockIdx.x;
    const int j0 = tj * TH, j1 = (tj == ntj - 1) ? g.N : j0 + TH;
    const int k0 = tk * TW, k1 = (tk == ntk - 1) ? g.K : k0 + TW;
    const int R1 = (MODE == 1) ? 1 : 0;
    const int jL0 = max(0, j0 - S - R1), jL1 = min(g.N, j1 + S + R1);
    const int kL0 = max(0, k0 - S - R1), kL1 = min(g.K, k1 + S + R1);
    STile<T> t = carve<T>(smem, jL0, kL0, jL1 - jL0, kL1 - kL0, g.f != nullptr);
    tile_load(g, t, zero_u != 0);
    if (prolong) {
        __syncthreads();
        // coarse block covering the tile, staged after the tile arrays
        const int cjA = jL0 >> 1, cjB = min(c.N - 1, ((jL1 - 1) >> 1) + 1);
        const int ckA = kL0 >> 1, ckB = min(c.K - 1, ((kL1 - 1) >> 1) + 1);
        const int EW = ckB - ckA + 1, EH = cjB - cjA + 1;
        T *E = t.cz + (t.LR + 1) * t.LC + (t.f ? t.LR * t.LC : 0);
        for (int i = threadIdx.x; i < EH * EW; i += blockDim.x) {
            const int rr = i / EW, cc = i - rr * EW;
            E[i] = c.u[(long)(cjA + rr) * c.P + ckA + cc];
        }
        __syncthreads();
        // u += P e (prolongate_kernel, :1034-1040), one fine node per thread
        const int n = t.LR * t.LC;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int r = i / t.LC, cc = i - r * t.LC;
            const int j = jL0 + r, k = kL0 + cc;
            if (k < 1 || k > g.K - 2 || j >= g.N - 1 + surface) continue;
            const T *e = E + ((j >> 1) - cjA) * EW + ((k >> 1) - ckA);
            T add;
            if (!(j & 1))
                add = (k & 1) ? (T)0.5 * (e[0] + e[1]) : e[0];
            else
                add = (k & 1) ? (T)0.25 * (e[0] + e[1] + e[EW] + e[EW + 1]) : (T)0.5 * (e[0] + e[EW]);
            t.u[i] += add;
        }
    }
    __syncthreads();
    for (int s = 0; s < S; s++) {
        tile_halfsweep(g, t, s & 1);
        __syncthreads();
    }
    const int ka = max(1, k0), kb = min(g.K - 2, k1 - 1);
    const int W = kb - ka + 1, n = (j1 - j0) * max(W, 0);
    double sq = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int rr = i / W, cc = i - rr * W;
        const int j = j0 + rr, k = ka + cc;
        const int li = (j - jL0) * t.LC + (k - kL0);
        if (MODE == 1) {
            const double rv = (double)tile_residual(g, t, j - jL0, k - kL0, j);
            sq += rv * rv;
        }
        if (MODE == 2)
            u64[(long)j * P64 + k] += (double)t.u[li];
        else
            g.u[(long)j * g.P + k] = t.u[li];
    }
    if (MODE == 1) {
        sq = block_sum_1d(sq);
        if (threadIdx.x == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = sq;
    }
}

// ---------------------------------------------------------------------------
// k_tail: levels l0 .. nlev-1 of the V-cycle in one CTA (global arrays,
// block barriers between phases).  Level l0's correction starts from zero.
// ---------------------------------------------------------------------------
struct TailLevels {
    int l0, nlev, nu_pre, nu_post, nu_coarse, surface;
};

template <typename T>
struct TailArgs {
    LvArgs<T> L[QD_MAXLEV];
    TailLevels p;
};

template <typename T>
__device__ void tail_halfsweep(const LvArgs<T> &g, int color, bool has_f) {
    const int HC = (g.K - 1) / 2;  // colour-compacted interior columns per row
    const int n = g.N * HC;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int j = i / HC, m = i - j * HC;
        const int k = 2 * m + 1 + ((j + 1 + color) & 1);
        if (k > g.K - 2) continue;
        const long c = (long)j * g.P + k;
        const long up = (j == 0) ? g.P : -(long)g.P;
        const long dn = (j == g.N - 1) ? -(long)g.P : g.P;
        T acc = g.cx[c - 1] * g.u[c - 1] + g.cx[c] * g.u[c + 1] + g.cz[c] * g.u[c + up] +
                g.cz[c + g.P] * g.u[c + dn];
        if (has_f) acc -= g.h2 * g.f[c];
        g.u[c] = g.dinv[c] * acc;
    }
}

template <typename T>
__device__ void tail_smooth(const LvArgs<T> &g, int nsweeps) {
    for (int s = 0; s < nsweeps; s++) {
        tail_halfsweep(g, 0, true);
        __syncthreads();
        tail_halfsweep(g, 1, true);
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(NT_TAIL) k_tail(TailArgs<T> a) {
    const TailLevels &p = a.p;
    for (int l = p.l0; l < p.nlev; l++) {
        const LvArgs<T> &g = a.L[l];
        for (int i = threadIdx.x; i < g.N * g.K; i += blockDim.x) {
            const int j = i / g.K, k = i - j * g.K;
            g.u[(long)j * g.P + k] = (T)0;
        }
        __syncthreads();
        if (l == p.nlev - 1) {
            tail_smooth(g, p.nu_coarse);
            break;
        }
        tail_smooth(g, p.nu_pre);
        for (int i = threadIdx.x; i < g.N * g.K; i += blockDim.x) {
            const int j = i / g.K, k = i - j * g.K;
            if (k < 1 || k > g.K - 2) continue;
            const long c = (long)j * g.P + k;
            const long up = (j == 0) ? g.P : -(long)g.P;
            const long dn = (j == g.N - 1) ? -(long)g.P : g.P;
            const T cW = g.cx[c - 1], cE = g.cx[c], cN = g.cz[c], cS = g.cz[c + g.P];
            const T lap = cW * g.u[c - 1] + cE * g.u[c + 1] + cN * g.u[c + up] + cS * g.u[c + dn] -
                          (((cW + cE) + cN) + cS) * g.u[c];
            g.r[c] = g.f[c] - lap * g.inv_h2;
        }
        __syncthreads();
        const LvArgs<T> &cl = a.L[l + 1];
        for (int i = threadIdx.x; i < cl.N * cl.K; i += blockDim.x) {
            const int j = i / cl.K, k = i - j * cl.K;
            if (k < 1 || k > cl.K - 2) continue;
            const int rn = (j == 0) ? 2 * j + 1 : 2 * j - 1;
            const int rs = (j == cl.N - 1) ? 2 * j - 1 : 2 * j + 1;
            const T *c0 = g.r + (long)(2 * j) * g.P + 2 * k;
            const T *cn = g.r + (long)rn * g.P + 2 * k;
            const T *cs = g.r + (long)rs * g.P + 2 * k;
            ((T *)cl.f)[(long)j * cl.P + k] =
                (T)0.06250 * ((T)4.0 * c0[0] + (T)2.0 * c0[-1] + (T)2.0 * c0[1] + (T)2.0 * cn[0] +
                              (T)2.0 * cs[0] + cn[-1] + cn[1] + cs[-1] + cs[1]);
        }
        __syncthreads();
    }
    for (int l = p.nlev - 2; l >= p.l0; l--) {
        const LvArgs<T> &g = a.L[l];
        const LvArgs<T> &cl = a.L[l + 1];
        for (int i = threadIdx.x; i < g.N * g.K; i += blockDim.x) {
            const int jf = i / g.K, kf = i - jf * g.K;
            if (jf >= g.N - 1 + p.surface || kf < 1 || kf > g.K - 2) continue;
            const T *e = cl.u + (long)(jf >> 1) * cl.P + (kf >> 1);
            T add;
            if (!(jf & 1))
                add = (kf & 1) ? (T)0.5 * (e[0] + e[1]) : e[0];
            else
                add = (kf & 1) ? (T)0.25 * (e[0] + e[1] + e[cl.P] + e[cl.P + 1]) : (T)0.5 * (e[0] + e[cl.P]);
            g.u[(long)jf * g.P + kf] += add;
        }
        __syncthreads();
        tail_smooth(g, p.nu_post);
    }
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
static int cdivi(int a, int b) { return (a + b - 1) / b; }

// fine-tile edge for level dims (N rows): aim for >= ~150 CTAs, cap by smem
template <typename T>
static int tile_edge(int N) {
    int t = sizeof(T) == 4 ? 64 : 32;
    while (t > 16 && cdivi(N - 1, t) * cdivi(N - 1, t) < 144) t /= 2;
    return t;
}

static size_t g_smem_limit = 0;

static size_t smem_limit() {
    if (!g_smem_limit) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        g_smem_limit = v > 0 ? (size_t)v : 48 * 1024;
    }
    return g_smem_limit;
}

template <typename T>
static int launch_down(qd_solver *s, Level<T> *Ls, int l, int S, int zero_u) {
    const LvArgs<T> g = lv(s, Ls, l), c = lv(s, Ls, l + 1);
    int TE = tile_edge<T>(g.N);
    int CH = TE / 2, CW = (sizeof(T) == 4 ? TE : 2 * TE) / 2;
    const int ntj = std::max(1, (c.N - 1) / CH), ntk = std::max(1, (c.K - 1) / CW);
    // largest tile: the last one absorbs the remainder
    const int maxCH = c.N - (ntj - 1) * CH, maxCW = c.K - (ntk - 1) * CW;
    const int LR = std::min(g.N, 2 * maxCH + 2 * S + 3), LC = std::min(g.K, 2 * maxCW + 2 * S + 3);
    const size_t smem = tile_bytes(sizeof(T), LR, LC, g.f != nullptr);
    if (smem > smem_limit()) {
        set_error("k_down tile %dx%d needs %zu B of shared memory", LR, LC, smem);
        return QD_ERR_ARG;
    }
    QD_CUDA(cudaFuncSetAttribute(k_down<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_down<T><<<dim3(ntk, ntj), NT, smem, s->stream>>>(g, c, CH, CW, ntj, ntk, S, zero_u);
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

template <typename T, int MODE>
static int launch_up(qd_solver *s, Level<T> *Ls, int l, int S, int prolong, int zero_u,
                     double *u64 = nullptr, int P64 = 0, int *nblocks = nullptr) {
    const LvArgs<T> g = lv(s, Ls, l);
    const LvArgs<T> c = (l + 1 < s->nlev) ? lv(s, Ls, l + 1) : g;
    const int TE = tile_edge<T>(g.N);
    const int TH = TE, TW = sizeof(T) == 4 ? TE : 2 * TE;
    const int ntj = std::max(1, (g.N - 1) / TH), ntk = std::max(1, (g.K - 1) / TW);
    const int maxTH = g.N - (ntj - 1) * TH, maxTW = g.K - (ntk - 1) * TW;
    const int R1 = MODE == 1 ? 1 : 0;
    const int LR = std::min(g.N, maxTH + 2 * (S + R1)), LC = std::min(g.K, maxTW + 2 * (S + R1));
    size_t smem = tile_bytes(sizeof(T), LR, LC, g.f != nullptr);
    if (prolong) smem += sizeof(T) * (size_t)(LR / 2 + 2) * (LC / 2 + 2);
    if (smem > smem_limit()) {
        set_error("k_up tile %dx%d needs %zu B of shared memory", LR, LC, smem);
        return QD_ERR_ARG;
    }
    if (MODE == 1 && ntj * ntk > s->n_partial) {
        set_error("too many tiles for the partial-sum buffer");
        return QD_ERR_ARG;
    }
    QD_CUDA(cudaFuncSetAttribute(k_up<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_up<T, MODE><<<dim3(ntk, ntj), NT, smem, s->stream>>>(g, c, TH, TW, ntj, ntk, S, prolong,
                                                         s->opt.surface_prolong, zero_u, s->d_partial,
                                                         u64, P64);
    QD_LAUNCH_CHECK(s);
    if (nblocks) *nblocks = ntj * ntk;
    return QD_OK;
}

// nsweeps red+black sweeps on level l as tile passes of at most SMAX
// half-sweeps (the first pass may start from a zero guess)
template <typename T>
static int smooth_passes(qd_solver *s, Level<T> *Ls, int l, int nsweeps, int zero_u) {
    int left = 2 * nsweeps;
    bool first = true;
    while (left > 0) {
        const int S = std::min(SMAX, left);
        QD_TRY((launch_up<T, 0>(s, Ls, l, S, 0, first ? zero_u : 0)));
        first = false;
        left -= S;
    }
    return QD_OK;
}

template <typename T>
static int first_tail_level(const qd_solver *s) {
    int lt = s->nlev;
    for (int l = s->nlev - 1; l >= 1; l--) {
        if (s->dims[l].N <= TAIL_N && s->dims[l].K <= TAIL_N) lt = l; else break;
    }
    return lt;
}

// One V-cycle on hierarchy Ls.  zero0: level 0 starts from a zero guess.
// MODE of level 0's k_up: 1 = plain (with residual norm), 2 = add into u64.
template <typename T, int MODE0>
static int vcycle_fused(qd_solver *s, Level<T> *Ls, int zero0, int *nblocks) {
    const int nl = s->nlev;
    if (nl == 1) return smooth_passes<T>(s, Ls, 0, s->opt.nu_coarse, zero0);
    const int lt = first_tail_level<T>(s);
    // descend through the tiled levels
    for (int l = 0; l < lt && l < nl - 1; l++) {
        const int zero = (l == 0) ? zero0 : 1;
        const int S = 2 * s->opt.nu_pre;
        const int Sfirst = S > SMAX ? S - SMAX : 0;
        if (Sfirst) QD_TRY(smooth_passes<T>(s, Ls, l, Sfirst / 2, zero));
        QD_TRY(launch_down<T>(s, Ls, l, std::min(S, SMAX), Sfirst ? 0 : zero));
    }
    // coarse tail (or the coarsest level on its own)
    if (lt < nl) {
        TailArgs<T> ta;
        for (int l = 0; l < nl; l++) ta.L[l] = lv(s, Ls, l);
        ta.p.l0 = lt; ta.p.nlev = nl; ta.p.nu_pre = s->opt.nu_pre; ta.p.nu_post = s->opt.nu_post;
        ta.p.nu_coarse = s->opt.nu_coarse; ta.p.surface = s->opt.surface_prolong;
        k_tail<T><<<1, NT_TAIL, 0, s->stream>>>(ta);
        QD_LAUNCH_CHECK(s);
    } else {
        QD_TRY(smooth_passes<T>(s, Ls, nl - 1, s->opt.nu_coarse, 1));
    }
    // ascend
    for (int l = std::min(lt, nl - 1) - 1; l >= 0; l--) {
        const int S = 2 * s->opt.nu_post;
        const int S1 = std::min(S, SMAX);
        const int rest = S - S1;
        if (l == 0 && rest == 0) {
            QD_TRY((launch_up<T, MODE0>(s, Ls, 0, S1, 1, 0, s->L64[0].u, s->dims[0].P, nblocks)));
        } else {
            QD_TRY((launch_up<T, 0>(s, Ls, l, S1, 1, 0)));
            if (rest) {
                if (l == 0) {
                    // remaining sweeps, the last pass in MODE0
                    int left = rest;
                    while (left > SMAX) {
                        QD_TRY((launch_up<T, 0>(s, Ls, 0, SMAX, 0, 0)));
                        left -= SMAX;
                    }
                    QD_TRY((launch_up<T, MODE0>(s, Ls, 0, left, 0, 0, s->L64[0].u, s->dims[0].P,
                                                nblocks)));
                } else {
                    QD_TRY(smooth_passes<T>(s, Ls, l, rest / 2, 0));
                }
            }
        }
    }
    return QD_OK;
}

int vcycle64_norm(qd_solver *s, int *nblocks) { return vcycle_fused<double, 1>(s, s->L64, 0, nblocks); }

int vcycle32_into64(qd_solver *s) { return vcycle_fused<float, 2>(s, s->L32, 1, nullptr); }

}  // namespace qd
