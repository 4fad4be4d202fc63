// mg_tile.cuh -- shared-memory tile kernels of the fused V-cycle (included by
// mg_fused.cu).
//
// A CTA of NT threads stages one tile (core + halo) of u, the face moduli
// and f with TMA 2-D bulk loads (tma.cuh): one thread issues the copies for
// all arrays against one mbarrier.  The tile origin column is rounded down to
// a 16-byte boundary and every array is a box of BH x W elements with row
// pitch W.  Loops over the tile are warp-per-row, lane-per-column.  One colour
// of red-black Gauss-Seidel per half-sweep; a node is updated only where its
// four neighbours lie in the tile, and the halo is as wide as the number of
// half-sweeps, so the core ends exact.
//
// Tiles stage 1/diag with the other arrays: a division (or a correctly
// rounded reciprocal) per update costs more issue slots than one more
// shared-memory load, and the boxes are sized so two CTAs still fit per SM.
//
// No kernel writes the array its tiles load u from: a tile's halo overlaps
// its neighbours' cores, and a CTA that stored its smoothed core into the
// source array before a neighbour's TMA load landed would hand that
// neighbour a halo already swept (a race that makes results depend on CTA
// scheduling).  Each level has two arrays, u and the scratch r; every tile
// kernel loads u from one (`src_r`) and writes the other (`dst`), boundary
// columns included, so the Dirichlet data travel with the field.
#pragma once

#include "tma.cuh"

namespace qd {

#define TWARP ((int)(threadIdx.x >> 5))
#define TLANE ((int)(threadIdx.x & 31))
#define TNWARP ((int)(blockDim.x >> 5))

template <typename T>
struct TileCfg {
    static constexpr bool kDinv = true;                  // 1/diag staged (dv array)
    static constexpr int kAlign = 16 / (int)sizeof(T);   // elements per 16 bytes
};

// tensor maps of one level's arrays, boxes of W x BH (cz: W x BH+1); ur is
// the map of the level's scratch array r, the other source of u
struct TileMaps {
    CUtensorMap u, ur, f, cx, cz, dv;
    int W, BH;
};

template <typename T>
struct STile {
    T *u, *f, *cx, *cz, *dv;
    int jL0, kL0;    // global row / column of smem (0,0); kL0 is 16-byte aligned
    int LR, LC;      // rows / columns of the tile that lie inside the grid
    int W;           // smem row pitch (the TMA box width)
};

__host__ __device__ inline size_t pad128(size_t bytes) { return (bytes + 127) & ~(size_t)127; }

// TMA destinations must be 128-byte aligned in the shared window; the
// dynamic allocation carries 128 spare bytes so the base can be rounded up
static constexpr size_t kSmemSlack = 128;
__device__ __forceinline__ unsigned char *align_smem128(unsigned char *p) {
    return p + ((128u - (smem_u32(p) & 127u)) & 127u);
}

// layout: u | cx | cz (BH+1 rows) | f (if has_f) | dv (FP64 only), each
// 128-byte aligned
template <typename T>
__host__ __device__ inline size_t tile_bytes(int BH, int W, bool has_f) {
    const size_t a = pad128(sizeof(T) * (size_t)BH * W), cz = pad128(sizeof(T) * (size_t)(BH + 1) * W);
    return 2 * a + cz + (has_f ? a : 0) + (TileCfg<T>::kDinv ? a : 0);
}

template <typename T>
__device__ __forceinline__ STile<T> carve(unsigned char *raw, int jL0, int kL0, int LR, int LC, int BH,
                                          int W, bool has_f) {
    STile<T> t;
    t.jL0 = jL0; t.kL0 = kL0; t.LR = LR; t.LC = LC; t.W = W;
    const size_t a = pad128(sizeof(T) * (size_t)BH * W), cz = pad128(sizeof(T) * (size_t)(BH + 1) * W);
    unsigned char *p = raw;
    t.u = reinterpret_cast<T *>(p); p += a;
    t.cx = reinterpret_cast<T *>(p); p += a;
    t.cz = reinterpret_cast<T *>(p); p += cz;
    t.f = has_f ? reinterpret_cast<T *>(p) : nullptr;
    if (has_f) p += a;
    t.dv = TileCfg<T>::kDinv ? reinterpret_cast<T *>(p) : nullptr;
    return t;
}

// Stage the tile: tile_issue starts the copies, tile_wait waits for them
// (the threads may do independent work in between).  u is zero-filled
// instead of loaded when zero_u; f is zero-filled when the level has no
// right-hand side but the kernel keeps an array for it.  tile_wait returns
// false (in every thread) if the copies did not land.
template <typename T>
__device__ void tile_issue(const LvArgs<T> &g, const TileMaps &m, STile<T> &t, bool zero_u, bool src_r,
                           uint64_t *bar) {
    const int BH = m.BH, W = m.W;
    const bool load_f = t.f && g.f;
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        // every box lands in full (rows past the grid arrive as zeros), so the
        // transaction count is the sum of the box sizes
        const unsigned a = (unsigned)(sizeof(T) * BH * W);
        unsigned bytes = a + (unsigned)(sizeof(T) * (BH + 1) * W);   // cx, cz
        if (!zero_u) bytes += a;
        if (load_f) bytes += a;
        if (TileCfg<T>::kDinv) bytes += a;
        mbar_expect_tx(bar, bytes);
        if (!zero_u) tma_load_2d(t.u, src_r ? &m.ur : &m.u, t.kL0, t.jL0, bar);
        tma_load_2d(t.cx, &m.cx, t.kL0, t.jL0, bar);
        tma_load_2d(t.cz, &m.cz, t.kL0, t.jL0, bar);
        if (load_f) tma_load_2d(t.f, &m.f, t.kL0, t.jL0, bar);
        if (TileCfg<T>::kDinv) tma_load_2d(t.dv, &m.dv, t.kL0, t.jL0, bar);
    }
    const int n = BH * W;
    if (zero_u)
        for (int i = threadIdx.x; i < n; i += blockDim.x) t.u[i] = (T)0;
    if (t.f && !g.f)
        for (int i = threadIdx.x; i < n; i += blockDim.x) t.f[i] = (T)0;
}

__device__ __forceinline__ bool tile_wait(uint64_t *bar, unsigned *status) {
    const bool ok = mbar_wait(bar, 0);
    if (!ok && status) atomicOr(status, ST_TMA_TIMEOUT);
    return __syncthreads_and(ok) != 0;
}

template <typename T>
__device__ bool tile_load(const LvArgs<T> &g, const TileMaps &m, STile<T> &t, bool zero_u, bool src_r,
                          uint64_t *bar, unsigned *status) {
    tile_issue(g, m, t, zero_u, src_r, bar);
    return tile_wait(bar, status);
}

// one colour over the tile
template <typename T>
__device__ void tile_halfsweep(const LvArgs<T> &g, const STile<T> &t, int color) {
    const int cmax = min(t.LC - 2, g.K - 2 - t.kL0);
    for (int r = TWARP; r < t.LR; r += TNWARP) {
        const int j = t.jL0 + r;
        const int rn = (j == 0) ? r + 1 : r - 1;
        const int rs = (j == g.N - 1) ? r - 1 : r + 1;
        if (rn < 0 || rn >= t.LR || rs < 0 || rs >= t.LR) continue;
        const int p = (color + j + t.kL0) & 1;
        const int sr = r * t.W, sn = rn * t.W, ss = rs * t.W;
        for (int c = p + 2 * TLANE; c <= cmax; c += 64) {
            if (c < 1) continue;
            const int idx = sr + c;
            const T cW = t.cx[idx - 1], cE = t.cx[idx], cN = t.cz[idx], cS = t.cz[idx + t.W];
            T acc = cW * t.u[idx - 1] + cE * t.u[idx + 1] + cN * t.u[sn + c] + cS * t.u[ss + c];
            if (t.f) acc -= g.h2 * t.f[idx];
            t.u[idx] = t.dv[idx] * acc;
        }
    }
}

// The first (red) half-sweep from a zero field: every neighbour is zero, so
// the update is u = dinv (0 - h2 f) -- the same value the general update
// gives (all four products are zero), with no neighbour or face-modulus
// loads.  Only the field's sign of zero can differ (-0 here where f = 0).
template <typename T>
__device__ void tile_first_halfsweep_from_zero(const LvArgs<T> &g, const STile<T> &t) {
    const int cmax = min(t.LC - 2, g.K - 2 - t.kL0);
    for (int r = TWARP; r < t.LR; r += TNWARP) {
        const int j = t.jL0 + r;
        const int rn = (j == 0) ? r + 1 : r - 1;
        const int rs = (j == g.N - 1) ? r - 1 : r + 1;
        if (rn < 0 || rn >= t.LR || rs < 0 || rs >= t.LR) continue;
        const int p = (j + t.kL0) & 1;
        const int sr = r * t.W;
        for (int c = p + 2 * TLANE; c <= cmax; c += 64) {
            if (c < 1) continue;
            const int idx = sr + c;
            const T f = t.f ? t.f[idx] : (T)0;
            t.u[idx] = t.dv[idx] * ((T)0 - g.h2 * f);
        }
    }
}

// residual at local (r, c) of global row j (interior column, neighbours in tile)
template <typename T>
__device__ __forceinline__ T tile_residual(const LvArgs<T> &g, const STile<T> &t, int r, int c, int j) {
    const int rn = (j == 0) ? r + 1 : r - 1;
    const int rs = (j == g.N - 1) ? r - 1 : r + 1;
    const int idx = r * t.W + c;
    const T cW = t.cx[idx - 1], cE = t.cx[idx], cN = t.cz[idx], cS = t.cz[idx + t.W];
    const T lap = cW * t.u[idx - 1] + cE * t.u[idx + 1] + cN * t.u[rn * t.W + c] + cS * t.u[rs * t.W + c] -
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
__global__ void __launch_bounds__(NT, 2)
    k_down(LvArgs<T> g, LvArgs<T> c, const __grid_constant__ TileMaps maps, int CH, int CW, int ntj,
           int ntk, int S, int zero_u, int src_r, T *dst, unsigned *status, const int *gate) {
    pdl_trigger();
    pdl_wait();   // launched with programmatic serialization: the previous kernel's data first
    if (gate && !__ldcg(gate)) return;   // a solve that needs no cycle: this one is skipped
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    unsigned char *smem = align_smem128(smem_raw);
    const int tj = blockIdx.y, tk = blockIdx.x;
    const int cj0 = tj * CH, cj1 = (tj == ntj - 1) ? c.N : cj0 + CH;
    const int ck0 = tk * CW, ck1 = (tk == ntk - 1) ? c.K : ck0 + CW;
    const int jL0 = max(0, 2 * cj0 - 2 - S);
    const int kL0 = max(0, 2 * ck0 - 2 - S) & ~(TileCfg<T>::kAlign - 1);
    const int LR = min(maps.BH, g.N - jL0), LC = min(maps.W, g.K - kL0);
    // the residual goes into f (FP32 levels and FP64 coarse levels all have
    // one) or, on the FP64 level 0 with its zero right-hand side, into dv
    const bool has_f = g.f != nullptr;
    STile<T> t = carve<T>(smem, jL0, kL0, LR, LC, maps.BH, maps.W, has_f);
    if (!tile_load(g, maps, t, zero_u != 0, src_r != 0, &bar, status)) return;
    for (int s = 0; s < S; s++) {
        if (s == 0 && zero_u)
            tile_first_halfsweep_from_zero(g, t);
        else
            tile_halfsweep(g, t, s & 1);
        __syncthreads();
    }
    T *res = t.f ? t.f : t.dv;
    {   // residual on fine rows 2cj0-1 .. 2cj1-1, columns 2ck0-1 .. 2ck1-1; a
        // node's residual reads f only at that node, so overwriting f in place
        // is race-free; u and the moduli are only read here
        const int ja = max(0, 2 * cj0 - 1), jb = min(g.N - 1, 2 * cj1 - 1);
        const int ka = max(1, 2 * ck0 - 1), kb = min(g.K - 2, 2 * ck1 - 1);
        for (int j = ja + TWARP; j <= jb; j += TNWARP)
            for (int k = ka + TLANE; k <= kb; k += 32)
                res[(j - jL0) * t.W + (k - kL0)] = tile_residual(g, t, j - jL0, k - kL0, j);
    }
    __syncthreads();
    {   // restriction onto owned coarse nodes (restriction_kernel, :953-1015)
        const int ka = max(1, ck0), kb = min(c.K - 2, ck1 - 1);
        for (int j = cj0 + TWARP; j < cj1; j += TNWARP) {
            const int rn = (j == 0) ? 2 * j + 1 : 2 * j - 1;
            const int rs = (j == c.N - 1) ? 2 * j - 1 : 2 * j + 1;
            const T *R0 = res + (2 * j - jL0) * t.W - kL0;
            const T *RN = res + (rn - jL0) * t.W - kL0;
            const T *RS = res + (rs - jL0) * t.W - kL0;
            for (int k = ka + TLANE; k <= kb; k += 32) {
                const int f = 2 * k;
                const T val = (T)0.06250 * ((T)4.0 * R0[f] + (T)2.0 * R0[f - 1] + (T)2.0 * R0[f + 1] +
                                            (T)2.0 * RN[f] + (T)2.0 * RS[f] + RN[f - 1] + RN[f + 1] +
                                            RS[f - 1] + RS[f + 1]);
                ((T *)c.f)[(long)j * c.P + k] = val;
            }
        }
    }
    {   // smoothed fine u on the owned region, the boundary columns with it
        const int ja = 2 * cj0, jb = min(g.N, 2 * cj1);
        const int ka = 2 * ck0, kb = min(g.K, 2 * ck1);
        for (int j = ja + TWARP; j < jb; j += TNWARP) {
            const T *ur = t.u + (j - jL0) * t.W - kL0;
            T *gr = dst + (long)j * g.P;
            for (int k = ka + TLANE; k < kb; k += 32) gr[k] = ur[k];
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
__global__ void __launch_bounds__(NT, 2)
    k_up(LvArgs<T> g, LvArgs<T> c, const __grid_constant__ TileMaps maps, int TH, int TW, int ntj,
         int ntk, int S, int prolong, int surface, int zero_u, int src_r, T *dst, const T *cu,
         double *partial, double *u64, int P64, unsigned *status, const int *gate) {
    pdl_trigger();
    pdl_wait();   // launched with programmatic serialization: the previous kernel's data first
    if (gate && !__ldcg(gate)) return;   // a solve that needs no cycle: this one is skipped
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    unsigned char *smem = align_smem128(smem_raw);
    const int tj = blockIdx.y, tk = blockIdx.x;
    const int j0 = tj * TH, j1 = (tj == ntj - 1) ? g.N : j0 + TH;
    const int k0 = tk * TW, k1 = (tk == ntk - 1) ? g.K : k0 + TW;
    const int R1 = (MODE == 1) ? 1 : 0;
    const int jL0 = max(0, j0 - S - R1);
    const int kL0 = max(0, k0 - S - R1) & ~(TileCfg<T>::kAlign - 1);
    const int LR = min(maps.BH, g.N - jL0), LC = min(maps.W, g.K - kL0);
    STile<T> t = carve<T>(smem, jL0, kL0, LR, LC, maps.BH, maps.W, g.f != nullptr);
    tile_issue(g, maps, t, zero_u != 0, src_r != 0, &bar);
    // coarse block covering the tile, gathered while the tile copies fly
    const int jL1 = jL0 + LR, kL1 = kL0 + LC;
    const int cjA = jL0 >> 1, cjB = min(c.N - 1, ((jL1 - 1) >> 1) + 1);
    const int ckA = kL0 >> 1, ckB = min(c.K - 1, ((kL1 - 1) >> 1) + 1);
    const int EW = ckB - ckA + 1;
    T *E = reinterpret_cast<T *>(smem + tile_bytes<T>(maps.BH, maps.W, g.f != nullptr));
    if (prolong)
        for (int r = TWARP; r <= cjB - cjA; r += TNWARP)
            for (int cc = TLANE; cc < EW; cc += 32) E[r * EW + cc] = cu[(long)(cjA + r) * c.P + ckA + cc];
    const bool ok = tile_wait(&bar, status);
    if (!ok) {
        if (MODE == 1 && threadIdx.x == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = 0.0;
        return;
    }
    if (prolong) {
        // u += P e (prolongate_kernel, :1034-1040)
        for (int r = TWARP; r < LR; r += TNWARP) {
            const int j = jL0 + r;
            if (j >= g.N - 1 + surface) continue;
            const T *er = E + ((j >> 1) - cjA) * EW - ckA;
            for (int cc = TLANE; cc < LC; cc += 32) {
                const int k = kL0 + cc;
                if (k < 1 || k > g.K - 2) continue;
                const T *e = er + (k >> 1);
                T add;
                if (!(j & 1))
                    add = (k & 1) ? (T)0.5 * (e[0] + e[1]) : e[0];
                else
                    add = (k & 1) ? (T)0.25 * (e[0] + e[1] + e[EW] + e[EW + 1]) : (T)0.5 * (e[0] + e[EW]);
                t.u[r * t.W + cc] += add;
            }
        }
        __syncthreads();
    }
    for (int s = 0; s < S; s++) {
        if (s == 0 && zero_u && !prolong)
            tile_first_halfsweep_from_zero(g, t);
        else
            tile_halfsweep(g, t, s & 1);
        __syncthreads();
    }
    const int ka = max(1, k0), kb = min(g.K - 2, k1 - 1);
    if (MODE == 2) {
        // u64 += e: the loads of two rows x two columns go out before any
        // store, so each warp waits on memory once per four nodes; e is
        // widened on the integer pipes (f2d_exact), leaving the FP64 pipe
        // one addition per node
        for (int jb = j0 + TWARP; jb < j1; jb += 2 * TNWARP) {
            double a[2][2];
#pragma unroll
            for (int q = 0; q < 2; q++)
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int j = jb + q * TNWARP, k = ka + TLANE + 32 * h;
                    a[q][h] = (j < j1 && k <= kb) ? __ldcg(u64 + (long)j * P64 + k) : 0.0;
                }
#pragma unroll
            for (int q = 0; q < 2; q++)
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int j = jb + q * TNWARP, k = ka + TLANE + 32 * h;
                    if (j < j1 && k <= kb)
                        u64[(long)j * P64 + k] = a[q][h] + f2d_exact(t.u[(j - jL0) * t.W + (k - kL0)]);
                }
            for (int q = 0; q < 2; q++) {   // columns past 64 (wide tiles only)
                const int j = jb + q * TNWARP;
                if (j >= j1) break;
                for (int k = ka + TLANE + 64; k <= kb; k += 32)
                    u64[(long)j * P64 + k] += f2d_exact(t.u[(j - jL0) * t.W + (k - kL0)]);
            }
        }
        return;
    }
    double sq = 0.0;
    // the write-out covers the boundary columns too (the copy carries the
    // Dirichlet data to the other array); the residual only the interior
    const int wa = (k0 == 0) ? 0 : ka, wb = (k1 == g.K) ? g.K - 1 : kb;
    for (int j = j0 + TWARP; j < j1; j += TNWARP) {
        const int r = j - jL0;
        for (int k = wa + TLANE; k <= wb; k += 32) {
            const int cc = k - kL0;
            if (MODE == 1 && k >= ka && k <= kb) {
                const double rv = (double)tile_residual(g, t, r, cc, j);
                sq += rv * rv;
            }
            dst[(long)j * g.P + k] = t.u[r * t.W + cc];
        }
    }
    if (MODE == 1) {
        sq = block_sum_1d(sq);
        if (threadIdx.x == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = sq;
    }
}

}  // namespace qd
