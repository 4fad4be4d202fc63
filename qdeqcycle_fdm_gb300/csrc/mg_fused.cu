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
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

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

}  // namespace qd

#include "mg_tile.cuh"

namespace qd {

// ---------------------------------------------------------------------------
// k_tail: levels l0 .. nlev-1 of the V-cycle in one CTA, with the levels'
// u, f and r in shared memory (and, when they fit, the face moduli too;
// otherwise those are read through the read-only cache).  Level l0's
// correction starts from zero; its f comes from k_down of level l0-1 and its
// u goes back to global memory for k_up of level l0-1.
// ---------------------------------------------------------------------------
struct TailLevels {
    int l0, nlev, nu_pre, nu_post, nu_coarse, surface, coef_smem;
    int coarse_solve, nint;   // exact coarsest solve with the dense inverse ainv
};

template <typename T>
struct TailArgs {
    LvArgs<T> L[QD_MAXLEV];
    const T *ainv;
    TailLevels p;
};

template <typename T>
struct TV {                       // one tail level as the kernel sees it
    T *u, *f, *r;                 // shared memory, row pitch K
    const T *cx, *cz, *dinv;      // shared (pitch K) or global (pitch P)
    int N, K, CP;
    T h2, inv_h2;
};

// one colour, warp per row and lane per node of that colour (a tail level
// has at most 65 columns, so one pass of a warp covers a row)
template <typename T>
__device__ void tv_halfsweep(const TV<T> &g, int color) {
    for (int j = TWARP; j < g.N; j += TNWARP) {
        const int up = (j == 0) ? g.K : -g.K;
        const int dn = (j == g.N - 1) ? -g.K : g.K;
        for (int k = 1 + ((j + 1 + color) & 1) + 2 * TLANE; k <= g.K - 2; k += 64) {
            const int c = j * g.K + k, cc = j * g.CP + k;
            // the moduli may live in shared or in global memory: generic loads
            T acc = g.cx[cc - 1] * g.u[c - 1] + g.cx[cc] * g.u[c + 1] + g.cz[cc] * g.u[c + up] +
                    g.cz[cc + g.CP] * g.u[c + dn];
            acc -= g.h2 * g.f[c];
            g.u[c] = g.dinv[cc] * acc;
        }
    }
}

template <typename T>
__device__ void tv_smooth(const TV<T> &g, int nsweeps) {
    for (int s = 0; s < nsweeps; s++) {
        tv_halfsweep(g, 0);
        __syncthreads();
        tv_halfsweep(g, 1);
        __syncthreads();
    }
}

template <typename T>
static size_t tail_smem_bytes(const qd_solver *s, int l0, int coef_smem) {
    size_t n = 0;
    for (int l = l0; l < s->nlev; l++) {
        const size_t nk = (size_t)s->dims[l].N * s->dims[l].K;
        n += 3 * nk + (coef_smem ? 3 * nk + s->dims[l].K : 0);
    }
    return n * sizeof(T);
}

template <typename T>
__global__ void __launch_bounds__(NT_TAIL) k_tail(TailArgs<T> a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const TailLevels &p = a.p;
    __shared__ TV<T> V[QD_MAXLEV];   // per-level views, read by every thread
    T *ptr = reinterpret_cast<T *>(smem);
    for (int l = p.l0; l < p.nlev; l++) {
        const LvArgs<T> &g = a.L[l];
        TV<T> v;
        const int n = g.N * g.K;
        v.N = g.N; v.K = g.K; v.h2 = g.h2; v.inv_h2 = g.inv_h2;
        v.u = ptr; ptr += n;
        v.f = ptr; ptr += n;
        v.r = ptr; ptr += n;
        if (p.coef_smem) {
            T *cx = ptr; ptr += n;
            T *cz = ptr; ptr += n + g.K;
            T *dv = ptr; ptr += n;
            for (int j = TWARP; j <= g.N; j += TNWARP)
                for (int k = TLANE; k < g.K; k += 32) {
                    const long gi = (long)j * g.P + k;
                    const int i = j * g.K + k;
                    cz[i] = g.cz[gi];
                    if (j < g.N) {
                        cx[i] = g.cx[gi];
                        dv[i] = g.dinv[gi];
                    }
                }
            v.cx = cx; v.cz = cz; v.dinv = dv; v.CP = g.K;
        } else {
            v.cx = g.cx; v.cz = g.cz; v.dinv = g.dinv; v.CP = g.P;
        }
        if (threadIdx.x == 0) V[l] = v;
    }
    __syncthreads();
    {   // right-hand side of the first tail level
        const LvArgs<T> &g = a.L[p.l0];
        for (int j = TWARP; j < g.N; j += TNWARP)
            for (int k = TLANE; k < g.K; k += 32) V[p.l0].f[j * g.K + k] = g.f[(long)j * g.P + k];
    }
    for (int l = p.l0; l < p.nlev; l++) {
        const TV<T> &g = V[l];
        for (int i = threadIdx.x; i < g.N * g.K; i += blockDim.x) g.u[i] = (T)0;
        __syncthreads();
        if (l == p.nlev - 1) {
            if (p.coarse_solve) {
                // e = A^-1 f over the interior nodes, one row per thread
                const int KI = g.K - 2;
                for (int i = threadIdx.x; i < p.nint; i += blockDim.x) {
                    const T *row = a.ainv + (long)i * p.nint;
                    T acc = (T)0;
                    int m = 0;
                    for (int jm = 0; jm < g.N; jm++)
                        for (int km = 1; km <= KI; km++, m++) acc += row[m] * g.f[jm * g.K + km];
                    const int j = i / KI, k = i - j * KI + 1;
                    g.u[j * g.K + k] = acc;
                }
                __syncthreads();
            } else {
                tv_smooth(g, p.nu_coarse);
            }
            break;
        }
        tv_smooth(g, p.nu_pre);
        for (int j = TWARP; j < g.N; j += TNWARP) {
            const int up = (j == 0) ? g.K : -g.K;
            const int dn = (j == g.N - 1) ? -g.K : g.K;
            for (int k = 1 + TLANE; k <= g.K - 2; k += 32) {
                const int i = j * g.K + k, cc = j * g.CP + k;
                const T cW = g.cx[cc - 1], cE = g.cx[cc], cN = g.cz[cc], cS = g.cz[cc + g.CP];
                const T lap = cW * g.u[i - 1] + cE * g.u[i + 1] + cN * g.u[i + up] + cS * g.u[i + dn] -
                              (((cW + cE) + cN) + cS) * g.u[i];
                g.r[i] = g.f[i] - lap * g.inv_h2;
            }
        }
        __syncthreads();
        const TV<T> &cl = V[l + 1];
        for (int j = TWARP; j < cl.N; j += TNWARP) {
            const int rn = (j == 0) ? 2 * j + 1 : 2 * j - 1;
            const int rs = (j == cl.N - 1) ? 2 * j - 1 : 2 * j + 1;
            for (int k = 1 + TLANE; k <= cl.K - 2; k += 32) {
                const T *c0 = g.r + (2 * j) * g.K + 2 * k;
                const T *cn = g.r + rn * g.K + 2 * k;
                const T *cs = g.r + rs * g.K + 2 * k;
                cl.f[j * cl.K + k] = (T)0.06250 * ((T)4.0 * c0[0] + (T)2.0 * c0[-1] + (T)2.0 * c0[1] +
                                                   (T)2.0 * cn[0] + (T)2.0 * cs[0] + cn[-1] + cn[1] +
                                                   cs[-1] + cs[1]);
            }
        }
        __syncthreads();
    }
    for (int l = p.nlev - 2; l >= p.l0; l--) {
        const TV<T> &g = V[l];
        const TV<T> &cl = V[l + 1];
        const int jmax = g.N - 1 + p.surface;
        for (int jf = TWARP; jf < jmax; jf += TNWARP) {
            const T *er = cl.u + (jf >> 1) * cl.K;
            for (int kf = 1 + TLANE; kf <= g.K - 2; kf += 32) {
                const T *e = er + (kf >> 1);
                T add;
                if (!(jf & 1))
                    add = (kf & 1) ? (T)0.5 * (e[0] + e[1]) : e[0];
                else
                    add = (kf & 1) ? (T)0.25 * (e[0] + e[1] + e[cl.K] + e[cl.K + 1])
                                   : (T)0.5 * (e[0] + e[cl.K]);
                g.u[jf * g.K + kf] += add;
            }
        }
        __syncthreads();
        tv_smooth(g, p.nu_post);
    }
    {   // the first tail level's correction, for k_up of the level above
        const LvArgs<T> &g = a.L[p.l0];
        for (int j = TWARP; j < g.N; j += TNWARP)
            for (int k = TLANE; k < g.K; k += 32) g.u[(long)j * g.P + k] = V[p.l0].u[j * g.K + k];
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

// raise a kernel's dynamic shared-memory limit once, to the device maximum
template <typename K>
static int set_smem(K kernel, size_t bytes) {
    // kernels already raised, keyed by their address (kernels of one
    // signature share K, so a per-type static would not do)
    static std::vector<std::pair<const void *, size_t>> raised;
    static std::mutex mtx;
    std::lock_guard<std::mutex> lock(mtx);
    size_t done = 0;
    for (const auto &e : raised)
        if (e.first == (const void *)kernel) done = e.second;
    if (bytes <= done) return QD_OK;
    cudaFuncAttributes fa;
    QD_CUDA(cudaFuncGetAttributes(&fa, kernel));
    const size_t cap = smem_limit() - fa.sharedSizeBytes;   // static + dynamic <= opt-in limit
    if (bytes > cap) {
        set_error("kernel needs %zu B of dynamic shared memory, %zu available", bytes, cap);
        return QD_ERR_ARG;
    }
    QD_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap));
    QD_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    raised.emplace_back((const void *)kernel, cap);
    return QD_OK;
}

// tensor maps of a level's arrays for a W x BH box, cached per solver
struct TmaCache {
    struct Entry {
        int level, fp64, W, BH;
        TileMaps maps;
    };
    std::vector<Entry> v;
};

template <typename T>
static int tile_maps(qd_solver *s, Level<T> *Ls, int l, int W, int BH, const TileMaps **out) {
    if (!s->tma_cache) s->tma_cache = new TmaCache();
    TmaCache *tc = static_cast<TmaCache *>(s->tma_cache);
    const int fp64 = sizeof(T) == 8;
    for (const auto &e : tc->v)
        if (e.level == l && e.fp64 == fp64 && e.W == W && e.BH == BH) {
            *out = &e.maps;
            return QD_OK;
        }
    TmaCache::Entry e;
    memset(&e, 0, sizeof(e));
    e.level = l; e.fp64 = fp64; e.W = W; e.BH = BH;
    e.maps.W = W; e.maps.BH = BH;
    const LevelDims &d = s->dims[l];
    QD_TRY(make_tensor_map_2d(&e.maps.u, Ls[l].u, fp64, d.K, d.N, d.P, W, BH));
    QD_TRY(make_tensor_map_2d(&e.maps.cx, Ls[l].cx, fp64, d.K, d.N, d.P, W, BH));
    QD_TRY(make_tensor_map_2d(&e.maps.cz, Ls[l].cz, fp64, d.K, d.N + 1, d.P, W, BH + 1));
    if (Ls[l].f) QD_TRY(make_tensor_map_2d(&e.maps.f, Ls[l].f, fp64, d.K, d.N, d.P, W, BH));
    if (fp64) QD_TRY(make_tensor_map_2d(&e.maps.dv, Ls[l].dinv, fp64, d.K, d.N, d.P, W, BH));
    tc->v.push_back(e);
    *out = &tc->v.back().maps;
    return QD_OK;
}

static int round_up(int x, int a) { return (x + a - 1) / a * a; }

template <typename T>
static int launch_down(qd_solver *s, Level<T> *Ls, int l, int S, int zero_u) {
    const LvArgs<T> g = lv(s, Ls, l), c = lv(s, Ls, l + 1);
    int TE = tile_edge<T>(g.N);
    int CH = TE / 2, CW = (sizeof(T) == 4 ? TE : 2 * TE) / 2;
    const int ntj = std::max(1, (c.N - 1) / CH), ntk = std::max(1, (c.K - 1) / CW);
    // largest tile: the last one absorbs the remainder; the box covers it
    // plus the column rounding of the aligned origin
    const int maxCH = c.N - (ntj - 1) * CH, maxCW = c.K - (ntk - 1) * CW;
    const int A = TileCfg<T>::kAlign;
    const int BH = 2 * maxCH + 2 * S + 3, W = round_up(2 * maxCW + 2 * S + 3 + A - 1, A);
    const bool has_f = (g.f != nullptr) || sizeof(T) == 4;
    const size_t smem = tile_bytes<T>(BH, W, has_f) + kSmemSlack;
    if (BH > 256 || W > 256 || smem > smem_limit()) {
        set_error("k_down tile %dx%d (%zu B of shared memory) exceeds the TMA box or smem", BH, W, smem);
        return QD_ERR_ARG;
    }
    const TileMaps *maps = nullptr;
    QD_TRY(tile_maps<T>(s, Ls, l, W, BH, &maps));
    QD_TRY(set_smem(k_down<T>, smem));
    k_down<T><<<dim3(ntk, ntj), NT, smem, s->stream>>>(g, c, *maps, CH, CW, ntj, ntk, S, zero_u,
                                                       &s->d_status->flags);
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
    const int A = TileCfg<T>::kAlign;
    const int BH = maxTH + 2 * (S + R1), W = round_up(maxTW + 2 * (S + R1) + A - 1, A);
    size_t smem = tile_bytes<T>(BH, W, g.f != nullptr);
    if (prolong) smem += sizeof(T) * (size_t)(BH / 2 + 2) * (W / 2 + 2);
    smem += kSmemSlack;
    if (BH > 256 || W > 256 || smem > smem_limit()) {
        set_error("k_up tile %dx%d (%zu B of shared memory) exceeds the TMA box or smem", BH, W, smem);
        return QD_ERR_ARG;
    }
    if (MODE == 1 && ntj * ntk > s->n_partial) {
        set_error("too many tiles for the partial-sum buffer");
        return QD_ERR_ARG;
    }
    const TileMaps *maps = nullptr;
    QD_TRY(tile_maps<T>(s, Ls, l, W, BH, &maps));
    QD_TRY(set_smem(k_up<T, MODE>, smem));
    k_up<T, MODE><<<dim3(ntk, ntj), NT, smem, s->stream>>>(g, c, *maps, TH, TW, ntj, ntk, S, prolong,
                                                         s->opt.surface_prolong, zero_u, s->d_partial,
                                                         u64, P64, &s->d_status->flags);
    QD_LAUNCH_CHECK(s);
    if (nblocks) *nblocks = ntj * ntk;
    return QD_OK;
}

// host side of tma.cuh: cuTensorMapEncodeTiled through the runtime's
// driver entry point (no link against libcuda)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int make_tensor_map_2d(CUtensorMap *map, const void *base, bool fp64, int width, int height,
                       int pitch, int box_w, int box_h) {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        QD_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                                 &q));
        if (!p || q != cudaDriverEntryPointSuccess) {
            set_error("cuTensorMapEncodeTiled is not available from the driver");
            return QD_ERR_CUDA;
        }
        fn = (EncodeTiledFn)p;
    }
    const size_t esz = fp64 ? 8 : 4;
    if (!base || ((uintptr_t)base & 15) || (pitch * esz) % 16 || (box_w * esz) % 16 || box_w < 1 ||
        box_w > 256 || box_h < 1 || box_h > 256 || width < 1 || height < 1) {
        set_error("tensor map %dx%d pitch %d box %dx%d violates the TMA rules", width, height, pitch,
                  box_w, box_h);
        return QD_ERR_ARG;
    }
    const cuuint64_t dims[2] = {(cuuint64_t)width, (cuuint64_t)height};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch * esz};
    const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    const cuuint32_t es[2] = {1, 1};
    const CUresult r = fn(map, fp64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                          const_cast<void *>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return QD_ERR_CUDA;
    }
    return QD_OK;
}

void tma_cache_free(qd_solver *s) {
    delete static_cast<TmaCache *>(s->tma_cache);
    s->tma_cache = nullptr;
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
        ta.p.coarse_solve = s->opt.coarse_solve;
        ta.p.nint = s->n_cint;
        ta.ainv = sizeof(T) == 8 ? (const T *)s->d_ainv64 : (const T *)s->d_ainv32;
        if (ta.p.coarse_solve && (s->n_cint == 0 || !ta.ainv)) {
            set_error("coarse_solve needs a coarsest level of at most 1024 unknowns");
            return QD_ERR_ARG;
        }
        ta.p.coef_smem = tail_smem_bytes<T>(s, lt, 1) <= smem_limit();
        const size_t smem = tail_smem_bytes<T>(s, lt, ta.p.coef_smem);
        if (smem > smem_limit()) {
            set_error("coarse tail needs %zu B of shared memory", smem);
            return QD_ERR_ARG;
        }
        QD_TRY(set_smem(k_tail<T>, smem));
        k_tail<T><<<1, NT_TAIL, smem, s->stream>>>(ta);
        QD_LAUNCH_CHECK(s);
    } else {
        if (s->opt.coarse_solve) {
            set_error("coarse_solve needs the coarsest level in the single-CTA tail (<= 65 rows)");
            return QD_ERR_ARG;
        }
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
