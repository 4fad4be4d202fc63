// mg_tile.cuh -- shared-memory tile kernels of the fused V-cycle (included by
// mg_fused.cu).
//
// A CTA of NT threads stages one tile (core + halo) of u, the face moduli and
// f.  Loops over the tile are warp-per-row, lane-per-column, so rows and
// columns come straight from the thread index.  One colour of red-black
// Gauss-Seidel per half-sweep; a node is updated only where its four
// neighbours lie in the tile, and the halo is as wide as the number of
// half-sweeps, so the core ends exact.
//
// FP64 tiles stage 1/diag (a double division costs ~30 instructions on
// GB300's FP64 pipe); FP32 tiles recompute it with a correctly rounded
// reciprocal, which frees shared memory for two CTAs per SM.
#pragma once

namespace qd {

#define TWARP ((int)(threadIdx.x >> 5))
#define TLANE ((int)(threadIdx.x & 31))
#define TNWARP ((int)(blockDim.x >> 5))

template <typename T>
struct TileCfg {
    static constexpr bool kDinv = sizeof(T) == 8;
};

__device__ __forceinline__ float recip(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double recip(double x) { return 1.0 / x; }

template <typename T>
struct STile {
    T *u, *f, *cx, *cz, *dv;
    int jL0, kL0, LR, LC;
};

// layout: u | cx | cz (LR+1 rows) | f (if has_f) | dv (FP64 only)
template <typename T>
__device__ __forceinline__ STile<T> carve(unsigned char *raw, int jL0, int kL0, int LR, int LC,
                                          bool has_f) {
    STile<T> t;
    t.jL0 = jL0; t.kL0 = kL0; t.LR = LR; t.LC = LC;
    const int n = LR * LC;
    T *p = reinterpret_cast<T *>(raw);
    t.u = p; p += n;
    t.cx = p; p += n;
    t.cz = p; p += n + LC;
    t.f = has_f ? p : nullptr;
    if (has_f) p += n;
    t.dv = TileCfg<T>::kDinv ? p : nullptr;
    return t;
}

template <typename T>
__host__ __device__ inline size_t tile_elems(int LR, int LC, bool has_f) {
    const size_t n = (size_t)LR * LC;
    return n * (3 + (has_f ? 1 : 0) + (TileCfg<T>::kDinv ? 1 : 0)) + LC;
}

// stage the tile; f is zero-filled when the level has no right-hand side
// but the kernel wants the array (to hold the residual)
template <typename T>
__device__ void tile_load(const LvArgs<T> &g, STile<T> &t, bool zero_u) {
    for (int r = TWARP; r < t.LR; r += TNWARP) {
        const long gr = (long)(t.jL0 + r) * g.P + t.kL0;
        const int sr = r * t.LC;
        for (int c = TLANE; c < t.LC; c += 32) {
            t.u[sr + c] = zero_u ? (T)0 : g.u[gr + c];
            t.cx[sr + c] = g.cx[gr + c];
            if (t.f) t.f[sr + c] = g.f ? g.f[gr + c] : (T)0;
            if (TileCfg<T>::kDinv) t.dv[sr + c] = g.dinv[gr + c];
        }
    }
    for (int r = TWARP; r <= t.LR; r += TNWARP) {
        const long gr = (long)(t.jL0 + r) * g.P + t.kL0;
        for (int c = TLANE; c < t.LC; c += 32) t.cz[r * t.LC + c] = g.cz[gr + c];
    }
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
        const int sr = r * t.LC, sn = rn * t.LC, ss = rs * t.LC;
        for (int c = p + 2 * TLANE; c <= cmax; c += 64) {
            if (c < 1) continue;
            const int idx = sr + c;
            const T cW = t.cx[idx - 1], cE = t.cx[idx], cN = t.cz[idx], cS = t.cz[idx + t.LC];
            T acc = cW * t.u[idx - 1] + cE * t.u[idx + 1] + cN * t.u[sn + c] + cS * t.u[ss + c];
            if (t.f) acc -= g.h2 * t.f[idx];
            const T d = TileCfg<T>::kDinv ? t.dv[idx] : recip(((cW + cE) + cN) + cS);
            t.u[idx] = d * acc;
        }
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
__global__ void __launch_bounds__(NT, 2)
    k_down(LvArgs<T> g, LvArgs<T> c, int CH, int CW, int ntj, int ntk, int S, int zero_u) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tj = blockIdx.y, tk = blockIdx.x;
    const int cj0 = tj * CH, cj1 = (tj == ntj - 1) ? c.N : cj0 + CH;
    const int ck0 = tk * CW, ck1 = (tk == ntk - 1) ? c.K : ck0 + CW;
    const int jL0 = max(0, 2 * cj0 - 2 - S), jL1 = min(g.N, 2 * cj1 + S + 1);
    const int kL0 = max(0, 2 * ck0 - 2 - S), kL1 = min(g.K, 2 * ck1 + S + 1);
    // the residual goes into f (FP32 levels and FP64 coarse levels all have
    // one) or, on the FP64 level 0 with its zero right-hand side, into dv
    const bool has_f = (g.f != nullptr) || !TileCfg<T>::kDinv;
    STile<T> t = carve<T>(smem, jL0, kL0, jL1 - jL0, kL1 - kL0, has_f);
    tile_load(g, t, zero_u != 0);
    __syncthreads();
    for (int s = 0; s < S; s++) {
        tile_halfsweep(g, t, s & 1);
        __syncthreads();
    }
    T *res = t.f ? t.f : t.dv;
    {   // residual on fine rows 2cj0-1 .. 2cj1-1, columns 2ck0-1 .. 2ck1-1
        const int ja = max(0, 2 * cj0 - 1), jb = min(g.N - 1, 2 * cj1 - 1);
        const int ka = max(1, 2 * ck0 - 1), kb = min(g.K - 2, 2 * ck1 - 1);
        // a node's residual reads f only at that node, so overwriting f in
        // place is race-free; u and the moduli are only read here
        for (int j = ja + TWARP; j <= jb; j += TNWARP)
            for (int k = ka + TLANE; k <= kb; k += 32)
                res[(j - jL0) * t.LC + (k - kL0)] = tile_residual(g, t, j - jL0, k - kL0, j);
    }
    __syncthreads();
    {   // restriction onto owned coarse nodes (restriction_kernel, :953-1015)
        const int ka = max(1, ck0), kb = min(c.K - 2, ck1 - 1);
        for (int j = cj0 + TWARP; j < cj1; j += TNWARP) {
            const int rn = (j == 0) ? 2 * j + 1 : 2 * j - 1;
            const int rs = (j == c.N - 1) ? 2 * j - 1 : 2 * j + 1;
            const T *R0 = res + (2 * j - jL0) * t.LC - kL0;
            const T *RN = res + (rn - jL0) * t.LC - kL0;
            const T *RS = res + (rs - jL0) * t.LC - kL0;
            for (int k = ka + TLANE; k <= kb; k += 32) {
                const int f = 2 * k;
                const T val = (T)0.06250 * ((T)4.0 * R0[f] + (T)2.0 * R0[f - 1] + (T)2.0 * R0[f + 1] +
                                            (T)2.0 * RN[f] + (T)2.0 * RS[f] + RN[f - 1] + RN[f + 1] +
                                            RS[f - 1] + RS[f + 1]);
                ((T *)c.f)[(long)j * c.P + k] = val;
            }
        }
    }
    {   // smoothed fine u on the owned region
        const int ja = 2 * cj0, jb = min(g.N, 2 * cj1);
        const int ka = max(1, 2 * ck0), kb = min(g.K - 1, 2 * ck1);
        for (int j = ja + TWARP; j < jb; j += TNWARP) {
            const T *ur = t.u + (j - jL0) * t.LC - kL0;
            T *gr = g.u + (long)j * g.P;
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
    k_up(LvArgs<T> g, LvArgs<T> c, int TH, int TW, int ntj, int ntk, int S, int prolong,
         int surface, int zero_u, double *partial, double *u64, int P64) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tj = blockIdx.y, tk = blockIdx.x;
    const int j0 = tj * TH, j1 = (tj == ntj - 1) ? g.N : j0 + TH;
    const int k0 = tk * TW, k1 = (tk == ntk - 1) ? g.K : k0 + TW;
    const int R1 = (MODE == 1) ? 1 : 0;
    const int jL0 = max(0, j0 - S - R1), jL1 = min(g.N, j1 + S + R1);
    const int kL0 = max(0, k0 - S - R1), kL1 = min(g.K, k1 + S + R1);
    const int LR = jL1 - jL0, LC = kL1 - kL0;
    STile<T> t = carve<T>(smem, jL0, kL0, LR, LC, g.f != nullptr);
    tile_load(g, t, zero_u != 0);
    if (prolong) {
        // coarse block covering the tile, staged after the tile arrays
        const int cjA = jL0 >> 1, cjB = min(c.N - 1, ((jL1 - 1) >> 1) + 1);
        const int ckA = kL0 >> 1, ckB = min(c.K - 1, ((kL1 - 1) >> 1) + 1);
        const int EW = ckB - ckA + 1;
        T *E = reinterpret_cast<T *>(smem) + tile_elems<T>(LR, LC, g.f != nullptr);
        for (int r = TWARP; r <= cjB - cjA; r += TNWARP)
            for (int cc = TLANE; cc < EW; cc += 32) E[r * EW + cc] = c.u[(long)(cjA + r) * c.P + ckA + cc];
        __syncthreads();
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
                t.u[r * LC + cc] += add;
            }
        }
    }
    __syncthreads();
    for (int s = 0; s < S; s++) {
        tile_halfsweep(g, t, s & 1);
        __syncthreads();
    }
    const int ka = max(1, k0), kb = min(g.K - 2, k1 - 1);
    double sq = 0.0;
    for (int j = j0 + TWARP; j < j1; j += TNWARP) {
        const int r = j - jL0;
        for (int k = ka + TLANE; k <= kb; k += 32) {
            const int cc = k - kL0;
            if (MODE == 1) {
                const double rv = (double)tile_residual(g, t, r, cc, j);
                sq += rv * rv;
            }
            if (MODE == 2)
                u64[(long)j * P64 + k] += (double)t.u[r * LC + cc];
            else
                g.u[(long)j * g.P + k] = t.u[r * LC + cc];
        }
    }
    if (MODE == 1) {
        sq = block_sum_1d(sq);
        if (threadIdx.x == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = sq;
    }
}

}  // namespace qd
