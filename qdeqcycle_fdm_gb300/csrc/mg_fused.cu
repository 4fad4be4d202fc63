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
// u, f and r in shared memory.  Their face moduli and the dense coarsest
// inverse never change, so they are packed once, at set-up, into one
// contiguous image in global memory laid out as the kernel uses them (row
// pitch K).  The kernel stages the longest prefix of the image that fits in
// shared memory with bulk asynchronous copies on one mbarrier, while its
// threads load f and clear u; arrays past the prefix are read in place.
// The image starts with the inverse and then holds the levels from the
// coarsest up, so the most-read arrays are the staged ones.  Level l0's
// correction starts from zero; its f comes from k_down of level l0-1 and
// its u goes back to global memory for k_up of level l0-1.
// ---------------------------------------------------------------------------
struct TailLevels {
    int l0, nlev, nu_pre, nu_post, nu_coarse, surface;
    int coarse_solve, nint;        // exact coarsest solve with the dense inverse
    int img_smem;                  // bytes of the image prefix staged in shared memory
    int work_off;                  // byte offset of the u/f/r arrays in shared memory
    int coef_off[QD_MAXLEV];       // element offset of level l's cx in the image (cz, dinv follow)
    int ainv_off;                  // element offset of the inverse (-1: none)
};

template <typename T>
struct TailArgs {
    LvArgs<T> L[QD_MAXLEV];
    const T *img;                  // the packed image in global memory
    unsigned *status;
    const int *gate;               // non-null: skip the launch when *gate is 0
    TailLevels p;
};

// element counts of a level's arrays in the image, each padded to 16 bytes
template <typename T>
__host__ __device__ inline int img_pad(long n) {
    const int a = 16 / (int)sizeof(T);
    return (int)((n + a - 1) / a * a);
}

// layout of the image: [inverse] then, for l = nlev-1 down to l0, cx | cz | dinv
template <typename T>
static size_t tail_layout(const qd_solver *s, int l0, TailLevels *p) {
    long off = 0;
    p->ainv_off = -1;
    if (s->n_cint > 0) {
        p->ainv_off = 0;
        off += img_pad<T>((long)s->n_cint * s->n_cint);
    }
    for (int l = s->nlev - 1; l >= l0; l--) {
        const long N = s->dims[l].N, K = s->dims[l].K;
        p->coef_off[l] = (int)off;
        off += img_pad<T>(N * K) + img_pad<T>((N + 1) * K) + img_pad<T>(N * K);
    }
    return (size_t)off * sizeof(T);
}

template <typename T>
struct TV {                       // one tail level as the kernel sees it
    T *u, *f, *r;                 // shared memory, row pitch K
    const T *cx, *cz, *dinv;      // shared or global (the image), row pitch K
    int N, K;
    T h2, inv_h2;
    int ou, of, orr, ocx, ocz, odv;   // the same arrays as element offsets in shared memory
};

// When every array of the tail is in shared memory the views are rebuilt
// from offsets against the kernel's own shared-memory base, so that the
// compiler sees shared-space pointers and issues shared-memory loads (a
// pointer read back from a struct is generic, and generic loads wait on the
// long scoreboard even when they hit shared memory).
template <typename T, bool ALLS>
__device__ __forceinline__ TV<T> tv_local(TV<T> v, T *sb) {
    if (ALLS) {
        v.u = sb + v.ou; v.f = sb + v.of; v.r = sb + v.orr;
        v.cx = sb + v.ocx; v.cz = sb + v.ocz; v.dinv = sb + v.odv;
    }
    return v;
}

// one colour, warp per row and lane per node of that colour (a tail level
// has at most 65 columns, so one pass of a warp covers a row)
template <typename T>
__device__ __forceinline__ void tv_halfsweep(const TV<T> &g, int color) {
    for (int j = TWARP; j < g.N; j += TNWARP) {
        const int up = (j == 0) ? g.K : -g.K;
        const int dn = (j == g.N - 1) ? -g.K : g.K;
        for (int k = 1 + ((j + 1 + color) & 1) + 2 * TLANE; k <= g.K - 2; k += 64) {
            const int c = j * g.K + k;
            // the moduli may live in shared or in global memory: generic loads
            T acc = g.cx[c - 1] * g.u[c - 1] + g.cx[c] * g.u[c + 1] + g.cz[c] * g.u[c + up] +
                    g.cz[c + g.K] * g.u[c + dn];
            acc -= g.h2 * g.f[c];
            g.u[c] = g.dinv[c] * acc;
        }
    }
}

template <typename T>
__device__ __forceinline__ void tv_smooth(const TV<T> &g, int nsweeps) {
    for (int s = 0; s < nsweeps; s++) {
        tv_halfsweep(g, 0);
        __syncthreads();
        tv_halfsweep(g, 1);
        __syncthreads();
    }
}

template <typename T>
static size_t tail_work_bytes(const qd_solver *s, int l0) {
    size_t n = 0;
    for (int l = l0; l < s->nlev; l++) n += 3 * (size_t)s->dims[l].N * s->dims[l].K;
    return n * sizeof(T);
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

template <typename T, bool ALLS>
__global__ void __launch_bounds__(NT_TAIL) k_tail(TailArgs<T> a) {
    pdl_trigger();
    pdl_wait();   // launched with programmatic serialization: the previous kernel's data first
    if (a.gate && !__ldcg(a.gate)) return;   // a solve that needs no cycle: this one is skipped
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ TV<T> V[QD_MAXLEV];   // per-level views, read by every thread
    __shared__ const T *ainv;
    unsigned char *smem = align_smem128(smem_raw);
    T *sb = reinterpret_cast<T *>(smem);
    const TailLevels &p = a.p;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        if (p.img_smem > 0) {
            mbar_expect_tx(&bar, (unsigned)p.img_smem);
            const int CH = 32768;
            for (int off = 0; off < p.img_smem; off += CH)
                bulk_load(smem + off, reinterpret_cast<const unsigned char *>(a.img) + off,
                          (unsigned)min(CH, p.img_smem - off), &bar);
        }
        // an array is read from shared memory when it lies inside the prefix
        const T *simg = reinterpret_cast<const T *>(smem);
        const long staged = p.img_smem / (long)sizeof(T);
        auto pick = [&](long off, long n) { return off + n <= staged ? simg + off : a.img + off; };
        T *w = reinterpret_cast<T *>(smem + p.work_off);
        for (int l = p.l0; l < p.nlev; l++) {
            const LvArgs<T> &g = a.L[l];
            const long N = g.N, K = g.K, n = N * K;
            TV<T> v;
            v.N = g.N; v.K = g.K; v.h2 = g.h2; v.inv_h2 = g.inv_h2;
            v.u = w; w += n;
            v.f = w; w += n;
            v.r = w; w += n;
            const long ox = p.coef_off[l], oz = ox + img_pad<T>(n), od = oz + img_pad<T>(n + K);
            v.cx = pick(ox, n);
            v.cz = pick(oz, n + K);
            v.dinv = pick(od, n);
            v.ou = (int)(v.u - sb); v.of = (int)(v.f - sb); v.orr = (int)(v.r - sb);
            v.ocx = (int)ox; v.ocz = (int)oz; v.odv = (int)od;
            V[l] = v;
        }
        ainv = p.ainv_off >= 0 ? pick(p.ainv_off, (long)p.nint * p.nint) : nullptr;
    }
    __syncthreads();
    {   // right-hand side of the first tail level; every correction starts at zero
        const LvArgs<T> &g = a.L[p.l0];
        const T *__restrict__ gf = g.f;
        T *sf = tv_local<T, ALLS>(V[p.l0], sb).f;
        for (int j = TWARP; j < g.N; j += TNWARP)
            for (int k = TLANE; k < g.K; k += 32) sf[j * g.K + k] = __ldg(gf + (long)j * g.P + k);
        for (int l = p.l0; l < p.nlev; l++) {
            const TV<T> v = tv_local<T, ALLS>(V[l], sb);
            for (int i = threadIdx.x; i < v.N * v.K; i += blockDim.x) v.u[i] = (T)0;
        }
    }
    bool ok = true;
    if (p.img_smem > 0) ok = mbar_wait(&bar, 0);
    if (!__syncthreads_and(ok)) {
        if (threadIdx.x == 0 && a.status) atomicOr(a.status, ST_TMA_TIMEOUT);
        return;
    }
    for (int l = p.l0; l < p.nlev; l++) {
        const TV<T> g = tv_local<T, ALLS>(V[l], sb);   // by value: stores through g.u cannot clobber it
        if (l == p.nlev - 1) {
            if (p.coarse_solve) {
                // e = A^-1 f over the interior nodes: a warp per row of the
                // inverse, lanes along the row, then a butterfly sum
                const int KI = g.K - 2;
                const T *ai = ALLS ? sb + p.ainv_off : ainv;
                for (int i = TWARP; i < p.nint; i += TNWARP) {
                    const T *row = ai + (long)i * p.nint;
                    T acc = (T)0;
                    for (int m = TLANE; m < p.nint; m += 32) {
                        const int jm = m / KI, km = m - jm * KI + 1;
                        acc += row[m] * g.f[jm * g.K + km];
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                    if (TLANE == 0) {
                        const int j = i / KI, k = i - j * KI + 1;
                        g.u[j * g.K + k] = acc;
                    }
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
                const int i = j * g.K + k;
                const T cW = g.cx[i - 1], cE = g.cx[i], cN = g.cz[i], cS = g.cz[i + g.K];
                const T lap = cW * g.u[i - 1] + cE * g.u[i + 1] + cN * g.u[i + up] + cS * g.u[i + dn] -
                              (((cW + cE) + cN) + cS) * g.u[i];
                g.r[i] = g.f[i] - lap * g.inv_h2;
            }
        }
        __syncthreads();
        const TV<T> cl = tv_local<T, ALLS>(V[l + 1], sb);
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
        const TV<T> g = tv_local<T, ALLS>(V[l], sb);
        const TV<T> cl = tv_local<T, ALLS>(V[l + 1], sb);
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
        const T *su = tv_local<T, ALLS>(V[p.l0], sb).u;
        for (int j = TWARP; j < g.N; j += TNWARP)
            for (int k = TLANE; k < g.K; k += 32) g.u[(long)j * g.P + k] = su[j * g.K + k];
    }
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
static int cdivi(int a, int b) { return (a + b - 1) / b; }


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
    QD_TRY(make_tensor_map_2d(&e.maps.ur, Ls[l].r, fp64, d.K, d.N, d.P, W, BH));
    QD_TRY(make_tensor_map_2d(&e.maps.cx, Ls[l].cx, fp64, d.K, d.N, d.P, W, BH));
    QD_TRY(make_tensor_map_2d(&e.maps.cz, Ls[l].cz, fp64, d.K, d.N + 1, d.P, W, BH + 1));
    if (Ls[l].f) QD_TRY(make_tensor_map_2d(&e.maps.f, Ls[l].f, fp64, d.K, d.N, d.P, W, BH));
    QD_TRY(make_tensor_map_2d(&e.maps.dv, Ls[l].dinv, fp64, d.K, d.N, d.P, W, BH));
    tc->v.push_back(e);
    *out = &tc->v.back().maps;
    return QD_OK;
}

static int round_up(int x, int a) { return (x + a - 1) / a * a; }

// Tile geometry.  A warp updates one row of a tile per pass, a lane every
// other node, so a box 64 columns wide keeps all 32 lanes busy in one pass
// per row; tile widths are chosen for W <= 64 and tile heights for about a
// full wave of CTAs at two CTAs per SM.
struct TileGeom {
    int ntj, ntk;     // tiles along rows / columns
    int BH, W;        // the staged box (largest over the tiles)
    int TH, TW;       // core rows / columns (fine nodes for k_up, coarse for k_down)
    size_t smem;
};

static constexpr int kBoxW = 64;       // default k_up boxes: one pass of 32 lanes per row
static constexpr int kDownBoxW = 64;   // default k_down boxes (qd_autotune may pick others)
// k_down's default box width: 64 columns, 128 on levels of 2049 columns or
// more, where the halo's share matters more than a wave's fill (measured at
// 4097^2: 203 us per launch with 128-column boxes, 207 with 64, 213 with 96),
// and 96 on FP32 levels of 1025 to 2048 columns (at 1025^2 in the rupture
// window: 16.7 us per launch against 19.1 with 64 and 20.2 with 80)
template <typename T>
static int down_box_default(int K) {
    if (K >= 2049) return 128;
    return (sizeof(T) == 4 && K >= 1025) ? 96 : kDownBoxW;
}
static constexpr int kWaveCtas = 150;

static size_t two_cta_smem() { return std::min<size_t>(smem_limit(), 112 * 1024); }

// k_up / smoother tiles on an N x K level with halo H: rows in blocks of TH
// (the last absorbs the remainder), columns in blocks of TW (the last is
// the short one).  Must match the tile bounds k_up computes.
static TileGeom up_geom(int N, int K, int TH, int TW, int H, int A) {
    TileGeom t{};
    t.TH = TH; t.TW = TW;
    t.ntj = std::max(1, (N - 1) / TH);
    t.ntk = std::max(1, cdivi(K - 1, TW));
    for (int tj = 0; tj < t.ntj; tj++) {
        const int j0 = tj * TH, j1 = (tj == t.ntj - 1) ? N : j0 + TH;
        t.BH = std::max(t.BH, std::min(N, j1 + H) - std::max(0, j0 - H));
    }
    for (int tk = 0; tk < t.ntk; tk++) {
        const int k0 = tk * TW, k1 = (tk == t.ntk - 1) ? K : k0 + TW;
        t.W = std::max(t.W, std::min(K, k1 + H) - (std::max(0, k0 - H) & ~(A - 1)));
    }
    t.W = round_up(t.W, A);
    return t;
}

// k_down tiles: coarse rows / columns in blocks of CH / CW over the coarse
// Nc x Kc level; the fine box spans rows 2cj0-2-S .. 2cj1+S.  Must match
// the tile bounds k_down computes.
static TileGeom down_geom(int Nc, int Kc, int N, int K, int CH, int CW, int S, int A) {
    TileGeom t{};
    t.TH = CH; t.TW = CW;
    t.ntj = std::max(1, (Nc - 1) / CH);
    t.ntk = std::max(1, cdivi(Kc - 1, CW));
    for (int tj = 0; tj < t.ntj; tj++) {
        const int c0 = tj * CH, c1 = (tj == t.ntj - 1) ? Nc : c0 + CH;
        t.BH = std::max(t.BH, std::min(N, 2 * c1 + S + 1) - std::max(0, 2 * c0 - 2 - S));
    }
    for (int tk = 0; tk < t.ntk; tk++) {
        const int c0 = tk * CW, c1 = (tk == t.ntk - 1) ? Kc : c0 + CW;
        t.W = std::max(t.W, std::min(K, 2 * c1 + S + 1) - (std::max(0, 2 * c0 - 2 - S) & ~(A - 1)));
    }
    t.W = round_up(t.W, A);
    return t;
}

template <typename T>
static size_t up_smem(const TileGeom &t, bool has_f, bool prolong) {
    size_t b = tile_bytes<T>(t.BH, t.W, has_f) + kSmemSlack;
    if (prolong) b += sizeof(T) * (size_t)(t.BH / 2 + 2) * (t.W / 2 + 2);
    return b;
}

// widest TW with W <= box, then the tallest TH that fits two CTAs per SM
// and still gives about a wave of CTAs
template <typename T>
static TileGeom pick_up(int N, int K, int H, bool has_f, bool prolong, int box) {
    const int A = TileCfg<T>::kAlign;
    int tw = std::max(A, (box - 2 * H) / A * A);
    while (tw > A && up_geom(N, K, 8, tw, H, A).W > box) tw -= A;
    TileGeom best{};
    bool found = false;
    for (int th = 64; th >= 8; th /= 2) {
        TileGeom t = up_geom(N, K, th, tw, H, A);
        t.smem = up_smem<T>(t, has_f, prolong);
        if (t.smem > two_cta_smem() && th > 8) continue;
        best = t;
        found = true;
        if (t.ntj * t.ntk >= kWaveCtas) break;
    }
    if (!found) best = up_geom(N, K, 8, tw, H, A);
    best.smem = up_smem<T>(best, has_f, prolong);
    return best;
}

template <typename T>
static TileGeom pick_down(int Nc, int Kc, int N, int K, int S, bool has_f, int box) {
    const int A = TileCfg<T>::kAlign;
    int cw = std::max(2, (box - 2 * S - 3) / 2);
    while (cw > 2 && down_geom(Nc, Kc, N, K, 8, cw, S, A).W > box) cw--;
    TileGeom best{};
    for (int ch = 32; ch >= 4; ch /= 2) {
        TileGeom t = down_geom(Nc, Kc, N, K, ch, cw, S, A);
        t.smem = tile_bytes<T>(t.BH, t.W, has_f) + kSmemSlack;
        best = t;
        if (t.smem > two_cta_smem() && ch > 4) continue;
        if (t.ntj * t.ntk >= kWaveCtas) break;
    }
    return best;
}

// Where a level's current field lives: u, or its scratch r.  Every tile
// kernel reads one and writes the other (see mg_tile.cuh).
template <typename T>
static T *field(Level<T> *Ls, int l, bool in_r) { return in_r ? Ls[l].r : Ls[l].u; }

// pre-smoothing + residual + restriction on level l: loads u from r when
// *in_r (ignored with zero_u), writes the smoothed field to the other array
// and flips *in_r
template <typename T>
static int launch_down(qd_solver *s, Level<T> *Ls, int l, int S, int zero_u, bool *in_r) {
    const LvArgs<T> g = lv(s, Ls, l), c = lv(s, Ls, l + 1);
    // the residual goes into f, or into the dinv slot on the FP64 level 0
    const bool has_f = g.f != nullptr;
    const TileGeom t = pick_down<T>(c.N, c.K, g.N, g.K, S, has_f, s->box_down ? s->box_down : down_box_default<T>(g.K));
    const int BH = t.BH, W = t.W, CH = t.TH, CW = t.TW, ntj = t.ntj, ntk = t.ntk;
    const size_t smem = t.smem;
    if (BH > 256 || W > 256 || smem > smem_limit()) {
        set_error("k_down tile %dx%d (%zu B of shared memory) exceeds the TMA box or smem", BH, W, smem);
        return QD_ERR_ARG;
    }
    const TileMaps *maps = nullptr;
    QD_TRY(tile_maps<T>(s, Ls, l, W, BH, &maps));
    QD_TRY(set_smem(k_down<T>, smem));
    QD_CUDA(launch_pdl(true, k_down<T>, dim3(ntk, ntj), dim3(NT), smem, s->stream, g, c, *maps, CH, CW, ntj, ntk,
                       S, zero_u, (int)*in_r, field(Ls, l, !*in_r), &s->d_status->flags, s->cycle_gate));
    QD_LAUNCH_CHECK(s);
    *in_r = !*in_r;
    return QD_OK;
}

// prolongation (prolong = 1, the coarse correction read from r when
// coarse_in_r) + S half-sweeps on level l: loads u from r when *in_r,
// writes the other array and flips *in_r (MODE 2: adds into u64 instead
// and leaves *in_r); MODE 1 also leaves the residual norm partials
template <typename T, int MODE>
static int launch_up(qd_solver *s, Level<T> *Ls, int l, int S, int prolong, int zero_u, bool *in_r,
                     bool coarse_in_r = false, double *u64 = nullptr, int P64 = 0, int *nblocks = nullptr) {
    const LvArgs<T> g = lv(s, Ls, l);
    const LvArgs<T> c = (l + 1 < s->nlev) ? lv(s, Ls, l + 1) : g;
    const int R1 = MODE == 1 ? 1 : 0;
    const TileGeom t = pick_up<T>(g.N, g.K, S + R1, g.f != nullptr, prolong != 0, s->box_up ? s->box_up : kBoxW);
    const int BH = t.BH, W = t.W, TH = t.TH, TW = t.TW, ntj = t.ntj, ntk = t.ntk;
    const size_t smem = t.smem;
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
    const T *cu = (l + 1 < s->nlev) ? field(Ls, l + 1, coarse_in_r) : nullptr;
    QD_CUDA(launch_pdl(true, k_up<T, MODE>, dim3(ntk, ntj), dim3(NT), smem, s->stream, g, c, *maps, TH, TW, ntj,
                       ntk, S, prolong, s->opt.surface_prolong, zero_u, (int)*in_r, field(Ls, l, !*in_r), cu,
                       s->d_partial, u64, P64, &s->d_status->flags, s->cycle_gate));
    QD_LAUNCH_CHECK(s);
    if (MODE != 2) *in_r = !*in_r;
    if (nblocks) *nblocks = ntj * ntk;
    return QD_OK;
}

// host side of tma.cuh: cuTensorMapEncodeTiled through the runtime's
// driver entry point (no link against libcuda)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encode_tiled_2d(CUtensorMap *map, const void *base, int dtype, int esz, long width, long height,
                    long pitch_bytes, int box_w, int box_h, int swizzle) {
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
    const int sw_bytes = swizzle == CU_TENSOR_MAP_SWIZZLE_128B ? 128
                         : swizzle == CU_TENSOR_MAP_SWIZZLE_64B ? 64
                         : swizzle == CU_TENSOR_MAP_SWIZZLE_32B ? 32 : 0;
    if (!base || ((uintptr_t)base & 15) || pitch_bytes % 16 || ((long)box_w * esz) % 16 || box_w < 1 ||
        box_w > 256 || box_h < 1 || box_h > 256 || width < 1 || height < 1 ||
        (sw_bytes && (long)box_w * esz > sw_bytes)) {
        set_error("tensor map %ldx%ld pitch %ld B box %dx%d violates the TMA rules", width, height,
                  pitch_bytes, box_w, box_h);
        return QD_ERR_ARG;
    }
    const cuuint64_t dims[2] = {(cuuint64_t)width, (cuuint64_t)height};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    const cuuint32_t es[2] = {1, 1};
    const CUresult r = fn(map, (CUtensorMapDataType)dtype, 2, const_cast<void *>(base), dims, strides, box,
                          es, CU_TENSOR_MAP_INTERLEAVE_NONE, (CUtensorMapSwizzle)swizzle,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return QD_ERR_CUDA;
    }
    return QD_OK;
}

// staged box widths of the tile kernels (multiples of 16 columns, 32..256;
// 0 restores the default); the solve graph is rebuilt on the next solve
int tiles_set(qd_solver *s, int box_up, int box_down) {
    auto ok = [](int b) { return b == 0 || (b >= 32 && b <= 256 && b % 16 == 0); };
    if (!ok(box_up) || !ok(box_down)) {
        set_error("tile box widths must be 0 or multiples of 16 in 32..256");
        return QD_ERR_ARG;
    }
    QD_CUDA(cudaStreamSynchronize(s->stream));
    s->box_up = box_up;
    s->box_down = box_down;
    solve_graph_free(s);
    return QD_OK;
}

// the box widths the level-0 tile kernels use when none is set (the level-0
// V-cycle runs in FP32 in mixed precision)
void tiles_default_level0(const qd_solver *s, int *box_up, int *box_down) {
    const int K = s->dims[0].K;
    *box_up = kBoxW;
    *box_down = s->opt.precision == QD_PREC_MIXED ? down_box_default<float>(K) : down_box_default<double>(K);
}

int encode_tiled_3d(CUtensorMap *map, const void *base, int dtype, int esz, long d0, long d1, long d2,
                    long stride1_bytes, long stride2_bytes, int box0, int box1, int box2, int swizzle) {
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
    const int sw_bytes = swizzle == CU_TENSOR_MAP_SWIZZLE_128B ? 128
                         : swizzle == CU_TENSOR_MAP_SWIZZLE_64B ? 64
                         : swizzle == CU_TENSOR_MAP_SWIZZLE_32B ? 32 : 0;
    if (!base || ((uintptr_t)base & 15) || stride1_bytes % 16 || stride2_bytes % 16 || ((long)box0 * esz) % 16 ||
        box0 < 1 || box0 > 256 || box1 < 1 || box1 > 256 || box2 < 1 || box2 > 256 || d0 < 1 || d1 < 1 ||
        d2 < 1 || (sw_bytes && (long)box0 * esz > sw_bytes)) {
        set_error("tensor map %ldx%ldx%ld box %dx%dx%d violates the TMA rules", d0, d1, d2, box0, box1, box2);
        return QD_ERR_ARG;
    }
    const cuuint64_t dims[3] = {(cuuint64_t)d0, (cuuint64_t)d1, (cuuint64_t)d2};
    const cuuint64_t strides[2] = {(cuuint64_t)stride1_bytes, (cuuint64_t)stride2_bytes};
    const cuuint32_t box[3] = {(cuuint32_t)box0, (cuuint32_t)box1, (cuuint32_t)box2};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = fn(map, (CUtensorMapDataType)dtype, 3, const_cast<void *>(base), dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, (CUtensorMapSwizzle)swizzle,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled (3-D) failed (%d)", (int)r);
        return QD_ERR_CUDA;
    }
    return QD_OK;
}

int make_tensor_map_2d(CUtensorMap *map, const void *base, bool fp64, int width, int height,
                       int pitch, int box_w, int box_h) {
    const int esz = fp64 ? 8 : 4;
    return encode_tiled_2d(map, base, fp64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                           esz, width, height, (long)pitch * esz, box_w, box_h, CU_TENSOR_MAP_SWIZZLE_NONE);
}

void tma_cache_free(qd_solver *s) {
    delete static_cast<TmaCache *>(s->tma_cache);
    s->tma_cache = nullptr;
}

// passes of at most SMAX half-sweeps (whole sweeps) for nsweeps sweeps;
// one more when `even` and their number is odd (a pass then carries fewer)
static int pass_count(int nsweeps, bool even) {
    int n = (2 * nsweeps + SMAX - 1) / SMAX;
    if (even && (n & 1)) n++;
    return n;
}

// nsweeps red+black sweeps on level l as `npass` tile passes of whole
// sweeps (the first pass may start from a zero guess); each pass reads one
// of u, r and writes the other
template <typename T>
static int smooth_passes(qd_solver *s, Level<T> *Ls, int l, int nsweeps, int npass, int zero_u, bool *in_r) {
    int left = nsweeps;
    for (int p = 0; p < npass; p++) {
        const int sw = (left + (npass - p) - 1) / (npass - p);   // spread evenly, at most SMAX / 2
        QD_TRY((launch_up<T, 0>(s, Ls, l, 2 * sw, 0, p == 0 ? zero_u : 0, in_r)));
        left -= sw;
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

// the single-CTA coarse tail from level lt down
template <typename T>
static int launch_tail(qd_solver *s, Level<T> *Ls, int lt) {
    const int nl = s->nlev;
    TailArgs<T> ta;
    for (int l = 0; l < nl; l++) ta.L[l] = lv(s, Ls, l);
    ta.p.l0 = lt; ta.p.nlev = nl;
    ta.p.nu_pre = s->tail_sweeps > 0 ? s->tail_sweeps : s->opt.nu_pre;
    ta.p.nu_post = s->tail_sweeps > 0 ? s->tail_sweeps : s->opt.nu_post;
    ta.p.nu_coarse = s->opt.nu_coarse; ta.p.surface = s->opt.surface_prolong;
    ta.p.coarse_solve = s->opt.coarse_solve;
    ta.p.nint = s->n_cint;
    ta.img = static_cast<const T *>(s->d_tail_img[sizeof(T) == 8]);
    ta.status = &s->d_status->flags;
    ta.gate = s->cycle_gate;
    if (!ta.img || s->tail_l0 != lt) {
        set_error("coarse tail image missing");
        return QD_ERR_ARG;
    }
    const size_t img = tail_layout<T>(s, lt, &ta.p);
    if (ta.p.coarse_solve && ta.p.ainv_off < 0) {
        set_error("coarse_solve needs a coarsest level of at most 1024 unknowns");
        return QD_ERR_ARG;
    }
    // the work arrays always live in shared memory; the image prefix
    // takes what is left (static shared memory and alignment kept aside)
    const size_t budget = smem_limit() - 4096, work = tail_work_bytes<T>(s, lt);
    if (work > budget) {
        set_error("coarse tail needs %zu B of shared memory", work);
        return QD_ERR_ARG;
    }
    const size_t prefix = std::min(img, (budget - work) / 128 * 128);
    ta.p.img_smem = (int)prefix;
    ta.p.work_off = (int)prefix;
    const size_t smem = prefix + work + kSmemSlack;
    if (prefix == img) {   // every array in shared memory
        QD_TRY(set_smem(k_tail<T, true>, smem));
        QD_CUDA(launch_pdl(true, k_tail<T, true>, dim3(1), dim3(NT_TAIL), smem, s->stream, ta));
    } else {
        QD_TRY(set_smem(k_tail<T, false>, smem));
        QD_CUDA(launch_pdl(true, k_tail<T, false>, dim3(1), dim3(NT_TAIL), smem, s->stream, ta));
    }
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

// One V-cycle on hierarchy Ls.  zero0: level 0 starts from a zero guess.
// MODE of level 0's k_up: 1 = plain (with residual norm), 2 = add into u64.
template <typename T, int MODE0>
static int vcycle_fused(qd_solver *s, Level<T> *Ls, int zero0, int *nblocks) {
    const int nl = s->nlev;
    bool in_r[QD_MAXLEV] = {};      // where each level's field lives (u or its scratch r)
    if (nl == 1) {
        // an even number of passes leaves the field in u
        QD_TRY(smooth_passes<T>(s, Ls, 0, s->opt.nu_coarse, pass_count(s->opt.nu_coarse, true), zero0, &in_r[0]));
        return QD_OK;
    }
    const int lt = first_tail_level<T>(s);
    const int pre = std::max(0, s->opt.nu_pre - SMAX / 2);    // sweeps before the fused k_down
    const int post = std::max(0, s->opt.nu_post - SMAX / 2);  // sweeps after the fused k_up
    // level 0 of the FP64 hierarchy must end in u (it is the solution): the
    // passes there, plus k_down and k_up, must be an even number of flips
    int pre0 = pass_count(pre, false), post0 = pass_count(post, false);
    if (MODE0 == 1 && ((pre0 + post0) & 1)) post0 > 0 ? post0++ : pre0++;
    // descend through the tiled levels
    for (int l = 0; l < lt && l < nl - 1; l++) {
        const int zero = (l == 0) ? zero0 : 1;
        const int np = (l == 0) ? pre0 : pass_count(pre, false);
        if (pre) QD_TRY(smooth_passes<T>(s, Ls, l, pre, np, zero, &in_r[l]));
        QD_TRY(launch_down<T>(s, Ls, l, std::min(2 * s->opt.nu_pre, SMAX), pre ? 0 : zero, &in_r[l]));
    }
    // coarse tail (or the coarsest level on its own)
    if (lt < nl) {
        QD_TRY(launch_tail<T>(s, Ls, lt));            // writes u of level lt
        in_r[lt] = false;
    } else {
        if (s->opt.coarse_solve) {
            set_error("coarse_solve needs the coarsest level in the single-CTA tail (<= 65 rows)");
            return QD_ERR_ARG;
        }
        QD_TRY(smooth_passes<T>(s, Ls, nl - 1, s->opt.nu_coarse, pass_count(s->opt.nu_coarse, false), 1,
                                &in_r[nl - 1]));
    }
    // ascend
    for (int l = std::min(lt, nl - 1) - 1; l >= 0; l--) {
        const int S1 = std::min(2 * s->opt.nu_post, SMAX);
        const int np = (l == 0) ? post0 : pass_count(post, false);
        if (l == 0 && !post) {
            QD_TRY((launch_up<T, MODE0>(s, Ls, 0, S1, 1, 0, &in_r[0], in_r[1], s->L64[0].u, s->dims[0].P,
                                        nblocks)));
        } else {
            QD_TRY((launch_up<T, 0>(s, Ls, l, S1, 1, 0, &in_r[l], in_r[l + 1])));
            if (post) {
                if (l == 0) {
                    // the remaining sweeps, the last pass in MODE0
                    if (np > 1) QD_TRY(smooth_passes<T>(s, Ls, 0, post - post / np, np - 1, 0, &in_r[0]));
                    QD_TRY((launch_up<T, MODE0>(s, Ls, 0, 2 * (post / np), 0, 0, &in_r[0], false, s->L64[0].u,
                                                s->dims[0].P, nblocks)));
                } else {
                    QD_TRY(smooth_passes<T>(s, Ls, l, post, np, 0, &in_r[l]));
                }
            }
        }
    }
    if (MODE0 == 1 && in_r[0]) {
        set_error("V-cycle left the level-0 field in its scratch array");
        return QD_ERR_STATE;
    }
    return QD_OK;
}

int vcycle64_norm(qd_solver *s, int *nblocks) { return vcycle_fused<double, 1>(s, s->L64, 0, nblocks); }

int vcycle32_into64(qd_solver *s) { return vcycle_fused<float, 2>(s, s->L32, 1, nullptr); }

// The level-0 smoothing pass of the mixed solver (the correction after a
// V-cycle that left the residual near the threshold): SMAX half-sweeps on
// A e = r from e = 0, then u64 += e -- the level-0 k_up of a cycle without
// the prolongation, one launch.
int smooth32_into64(qd_solver *s) {
    bool in_r = false;
    return launch_up<float, 2>(s, s->L32, 0, SMAX, 0, 1, &in_r, false, s->L64[0].u, s->dims[0].P);
}

// One kernel of the V-cycle the solver's precision runs, launched `reps`
// times back to back on the solver's stream between two events: the
// per-launch time of a kernel that otherwise runs inside the solve graph.
// The launches change the solver's state (they smooth, restrict and add
// corrections), so this is for measurements after a run.
template <typename T, int MODE_UP>
static int time_kernel_t(qd_solver *s, Level<T> *Ls, int which, int reps) {
    const int S = std::min(2 * s->opt.nu_pre, SMAX), S1 = std::min(2 * s->opt.nu_post, SMAX);
    for (int i = 0; i < reps; i++) {
        switch (which) {
            case QD_KERNEL_DOWN0: {
                // as in a cycle: the FP64 solution in (the mixed solver's
                // FP32 correction starts from zero and loads no u), the
                // smoothed field into the scratch array
                bool in_r = false;
                QD_TRY(launch_down<T>(s, Ls, 0, S, MODE_UP == 2 ? 1 : 0, &in_r));
                break;
            }
            case QD_KERNEL_UP0: {
                // as in a cycle: the scratch array in, u (or u64 += e) out
                int nb = 0;
                bool in_r = true;
                QD_TRY((launch_up<T, MODE_UP>(s, Ls, 0, S1, 1, 0, &in_r, false, s->L64[0].u, s->dims[0].P, &nb)));
                break;
            }
            case QD_KERNEL_TAIL:
                if (s->tail_l0 >= s->nlev) {
                    set_error("this hierarchy has no coarse tail");
                    return QD_ERR_ARG;
                }
                QD_TRY(launch_tail<T>(s, Ls, s->tail_l0));
                break;
            default:
                set_error("unknown kernel id %d", which);
                return QD_ERR_ARG;
        }
    }
    return QD_OK;
}

int time_kernel(qd_solver *s, int which, int reps, double *us) {
    if (s->nlev < 2 || reps < 1) {
        set_error("time_kernel needs two levels and reps >= 1");
        return QD_ERR_ARG;
    }
    cudaEvent_t e0, e1;
    QD_CUDA(cudaEventCreate(&e0));
    QD_CUDA(cudaEventCreate(&e1));
    int rc = QD_OK;
    if (cudaEventRecord(e0, s->stream) != cudaSuccess) rc = QD_ERR_CUDA;
    if (rc == QD_OK) {
        if (which == QD_KERNEL_RESIDUAL)
            for (int i = 0; i < reps && rc == QD_OK; i++) rc = level0_norm(s, 1, 0);
        else if (s->opt.precision == QD_PREC_MIXED)
            rc = time_kernel_t<float, 2>(s, s->L32, which, reps);
        else
            rc = time_kernel_t<double, 1>(s, s->L64, which, reps);
    }
    float ms = 0.f;
    if (rc == QD_OK && (cudaEventRecord(e1, s->stream) != cudaSuccess ||
                        cudaEventSynchronize(e1) != cudaSuccess ||
                        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)) {
        set_error("time_kernel: event timing failed");
        rc = QD_ERR_CUDA;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == QD_OK) *us = 1e3 * ms / reps;
    return rc;
}

// pack one hierarchy's tail moduli (and the coarsest inverse) into its image
template <typename T>
static int build_image(qd_solver *s, const Level<T> *Ls, const T *ainv, void **out) {
    const int lt = s->tail_l0;
    TailLevels p;
    const size_t bytes = tail_layout<T>(s, lt, &p);
    T *img = nullptr;
    QD_CUDA(cudaMalloc(&img, bytes));
    *out = img;
    QD_CUDA(cudaMemsetAsync(img, 0, bytes, s->stream));
    if (p.ainv_off >= 0 && ainv)
        QD_CUDA(cudaMemcpyAsync(img + p.ainv_off, ainv, sizeof(T) * (size_t)s->n_cint * s->n_cint,
                                cudaMemcpyDeviceToDevice, s->stream));
    for (int l = lt; l < s->nlev; l++) {
        const LevelDims &d = s->dims[l];
        const long n = (long)d.N * d.K;
        T *cx = img + p.coef_off[l], *cz = cx + img_pad<T>(n), *dv = cz + img_pad<T>(n + d.K);
        const size_t w = sizeof(T) * d.K, sp = sizeof(T) * d.P;
        QD_CUDA(cudaMemcpy2DAsync(cx, w, Ls[l].cx, sp, w, d.N, cudaMemcpyDeviceToDevice, s->stream));
        QD_CUDA(cudaMemcpy2DAsync(cz, w, Ls[l].cz, sp, w, d.N + 1, cudaMemcpyDeviceToDevice, s->stream));
        QD_CUDA(cudaMemcpy2DAsync(dv, w, Ls[l].dinv, sp, w, d.N, cudaMemcpyDeviceToDevice, s->stream));
    }
    return QD_OK;
}

// Set-up of the coarse-tail images, once the moduli and the coarsest
// inverse exist (end of mg_alloc).
int tail_image_build(qd_solver *s) {
    s->tail_l0 = first_tail_level<float>(s);
    if (s->tail_l0 >= s->nlev) return QD_OK;
    QD_TRY(build_image<float>(s, s->L32, s->d_ainv32, &s->d_tail_img[0]));
    QD_TRY(build_image<double>(s, s->L64, s->d_ainv64, &s->d_tail_img[1]));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    return QD_OK;
}

void tail_image_free(qd_solver *s) {
    for (int i = 0; i < 2; i++) {
        cudaFree(s->d_tail_img[i]);
        s->d_tail_img[i] = nullptr;
    }
}


// The bounded wait of the staging pipelines, exercised where nothing can
// complete it: one thread initialises an mbarrier that expects one arrival,
// nothing arrives, and the wait gives up after `polls` polls and records
// ST_TMA_TIMEOUT in the status word, as a tile kernel whose staging never
// landed does.  No copy is in flight, so the kernel simply returns.
__global__ void k_wait_probe(unsigned polls, unsigned *status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    if (!mbar_wait_limit(&bar, 0, polls) && threadIdx.x == 0 && status) atomicOr(status, ST_TMA_TIMEOUT);
}

int wait_probe(qd_solver *s, unsigned polls) {
    k_wait_probe<<<1, 32, 0, s->stream>>>(polls, &s->d_status->flags);
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

}  // namespace qd
