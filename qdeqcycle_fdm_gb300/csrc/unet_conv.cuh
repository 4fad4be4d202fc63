// unet_conv.cuh -- 3x3 convolutions of the warm-start U-Net on tcgen05.
//
// Activations are BF16, NHWC, on a padded grid: H+2 rows of Wp >= W+2
// pixels (Wp a multiple of 8), the border pixels held at zero, flattened to
// P = (H+2)*Wp pixel rows of C channels.  With that layout a 3x3 tap (dy,dx)
// is a shift of the pixel index by dy*Wp + dx, so
//
//   out[p, n] = sum_t sum_c in[p + shift_t, c] * W[t][n][c]
//
// is nine accumulated GEMMs whose A operand is the activation tile shifted
// by whole pixel rows -- the TMA box origin moves along the outer (pixel)
// coordinate, which needs no alignment, and out-of-range rows arrive as
// zeros.  No im2col buffer exists.
//
// k_conv_fwd: one CTA per MT x 128 output pixels (MT sub-tiles sharing each
//   staged weight tile), N = Cout accumulator columns per sub-tile in tensor
//   memory.  K steps = 9 taps x (Cin / KB) channel blocks of
//   KB = min(Cin, 64) channels (rows of 32, 64 or 128 bytes, matching
//   swizzle).  Warp 0 lane 0 streams A/B tiles with TMA through a STAGES-deep
//   ring of mbarriers, warp 1 lane 0 issues the MMAs, warp 2 owns the tensor
//   memory, and all four warps run the epilogue (bias, ReLU, gradient mask,
//   border zeroing, BF16 or FP32 store).  The same kernel computes the data
//   gradient of a convolution, with the tap order reversed and the weights
//   transposed per tap.
// k_conv_wgrad: dW[t][co][ci] = sum_p dY[p, co] * X[p + shift_t, ci] with
//   pixel-contiguous (planar) copies of dY and X: M = Cout rows (padded to
//   128 by the TMA zero fill), N = Cin, K = a chunk of pixels; one CTA per
//   (chunk, tap) writes its partial product to part[chunk][t][co][ci], and
//   k_sum_parts adds the chunks in order: training is deterministic.
//   The X copies are pre-shifted by dx in {-1, 0, 1}, so the remaining tap
//   shift dy*Wp is a multiple of 8 pixels (16 bytes): a legal TMA x origin.
//
// Every wait is bounded; a wait that gives up records ST_UNET_TIMEOUT in the
// status word and the kernel winds down without further waits on copies it
// never issued.
#pragma once

#include "tc.cuh"

namespace qd {

static constexpr unsigned ST_UNET_TIMEOUT = 16u;
static constexpr int CONV_STAGES = 3;
static constexpr int CONV_THREADS = 128;

struct ConvArgs {
    int Cin, Cout, KB;        // channels; channel block per K step
    int Wp, H, W, P;          // padded grid: P = (H+2)*Wp pixels, interior 1..H x 1..W
    int relu;                 // apply ReLU
    const float *bias;        // Cout (nullable)
    __nv_bfloat16 *out;       // NHWC Cout (or null when out_f32 is set)
    float *out_f32;           // channel 0 only, P floats (nullable)
    const __nv_bfloat16 *mask;  // multiply by (mask > 0), NHWC Cout (nullable)
    int tap_reverse;          // data-gradient mode: tap t reads shift of tap 8-t
    unsigned *status;
};

__device__ __forceinline__ int cdiv_dev(int a, int b) { return (a + b - 1) / b; }

__device__ __forceinline__ int tap_shift(int t, int Wp) { return (t / 3 - 1) * Wp + (t % 3 - 1); }

__device__ __forceinline__ bool interior_pixel(int p, const ConvArgs &a) {
    const int r = p / a.Wp, c = p - r * a.Wp;
    return r >= 1 && r <= a.H && c >= 1 && c <= a.W;
}

// 128-row sub-tiles per CTA: the weights of a K step are staged once for MT
// pixel tiles, and the per-CTA set-up (barriers, tensor memory) is paid once
// per MT tiles; MT * COUT accumulator columns stay within 256
template <int KB, int COUT>
__host__ __device__ constexpr int conv_mt() {
    return (128 / KB) < (256 / COUT) ? (128 / KB) : (256 / COUT);
}

// MT_: sub-tiles per CTA (0: conv_mt's choice; 1 for grids too small to
// fill the GPU with MT-tile CTAs)
template <int KB, int COUT, int MT_ = 0>
__global__ void __launch_bounds__(CONV_THREADS) k_conv_fwd(const __grid_constant__ CUtensorMap ta,
                                                           const __grid_constant__ CUtensorMap tb,
                                                           ConvArgs a) {
    constexpr int MT = MT_ ? MT_ : conv_mt<KB, COUT>();
    constexpr int ROWB = KB * 2;                        // bytes per operand row
    constexpr int ATILE = 128 * ROWB, ABYTES = MT * ATILE, BBYTES = COUT * ROWB;
    constexpr int STAGE = ((ABYTES + BBYTES) + 1023) / 1024 * 1024;
    constexpr int NC = MT * COUT;
    constexpr uint32_t TCOLS = NC <= 32 ? 32 : (NC <= 64 ? 64 : (NC <= 128 ? 128 : 256));
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[CONV_STAGES], empty[CONV_STAGES], done;
    __shared__ uint32_t tmem_base;
    __shared__ float sbias[COUT];
    unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * 128 * MT;
    // the bias is a parameter of the layer: no kernel the forward pass
    // overlaps with writes it
    for (int i = threadIdx.x; i < COUT; i += blockDim.x) sbias[i] = a.bias ? a.bias[i] : 0.f;
    const int nkb = a.Cin / KB, nsteps = 9 * nkb;

    if (threadIdx.x == 0) {
        for (int s = 0; s < CONV_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&done, 1);
    }
    if (warp == 2) tmem_alloc(&tmem_base, TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    pdl_trigger();
    pdl_wait();          // the set-up above overlapped the previous kernel's tail

    if (warp == 0 && lane == 0) {
        // producer: MT activation tiles and one weight tile per K step
        for (int s = 0; s < nsteps; s++) {
            const int st = s % CONV_STAGES;
            if (s >= CONV_STAGES && !mbar_wait(&empty[st], ((s / CONV_STAGES) - 1) & 1)) {
                atomicOr(a.status, ST_UNET_TIMEOUT);
                break;
            }
            const int t = s / nkb, kb = s - t * nkb;
            const int sh = tap_shift(a.tap_reverse ? 8 - t : t, a.Wp);
            unsigned char *sa = smem + st * STAGE, *sb = sa + ABYTES;
            mbar_expect_tx(&full[st], ABYTES + BBYTES);
#pragma unroll
            for (int mt = 0; mt < MT; mt++)
                tma_load_2d(sa + mt * ATILE, &ta, kb * KB, m0 + mt * 128 + sh, &full[st]);
            tma_load_2d(sb, &tb, kb * KB, t * COUT, &full[st]);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: sub-tile mt accumulates into columns mt*COUT ..
        constexpr uint32_t idesc = idesc_bf16_f32(COUT);
        for (int s = 0; s < nsteps; s++) {
            const int st = s % CONV_STAGES;
            if (!mbar_wait(&full[st], (s / CONV_STAGES) & 1)) {
                atomicOr(a.status, ST_UNET_TIMEOUT);
                break;
            }
            tc_fence_after();
            const uint32_t sa = smem_u32(smem + st * STAGE), sb = sa + ABYTES;
#pragma unroll
            for (int mt = 0; mt < MT; mt++)
#pragma unroll
                for (int k = 0; k < KB / 16; k++)
                    mma_bf16(tmem + (uint32_t)(mt * COUT), smem_desc(sa + mt * ATILE + 32 * k, ROWB),
                             smem_desc(sb + 32 * k, ROWB), idesc, (s > 0 || k > 0) ? 1u : 0u);
            mma_commit(&empty[st]);
        }
        mma_commit(&done);
    }
    __syncwarp();
    // epilogue: thread (warp, lane) owns pixel m0 + 128*mt + 32*warp + lane
    const bool ok = mbar_wait(&done, 0);
    if (!ok && threadIdx.x == 0) atomicOr(a.status, ST_UNET_TIMEOUT);
    tc_fence_after();
#pragma unroll 1
    for (int mt = 0; mt < MT; mt++) {
        const int p = m0 + mt * 128 + 32 * warp + lane;
        const bool in = p < a.P && interior_pixel(p, a);
#pragma unroll
        for (int n0 = 0; n0 < COUT; n0 += 8) {
            float v[8];
            tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(mt * COUT + n0), v);
            if (p >= a.P || !ok) continue;
#pragma unroll
            for (int i = 0; i < 8; i++) {
                float x = v[i] + sbias[n0 + i];
                if (a.relu) x = fmaxf(x, 0.f);
                v[i] = x;
            }
            if (a.mask && in) {
                const uint4 mk = *reinterpret_cast<const uint4 *>(a.mask + (size_t)p * COUT + n0);
                const __nv_bfloat16 *mv = reinterpret_cast<const __nv_bfloat16 *>(&mk);
#pragma unroll
                for (int i = 0; i < 8; i++)
                    if (!(__bfloat162float(mv[i]) > 0.f)) v[i] = 0.f;
            }
            if (!in) {
#pragma unroll
                for (int i = 0; i < 8; i++) v[i] = 0.f;
            }
            if (a.out_f32) {
                if (n0 == 0) a.out_f32[p] = v[0];
            } else {
                uint4 o;
                __nv_bfloat162 *ov = reinterpret_cast<__nv_bfloat162 *>(&o);
#pragma unroll
                for (int i = 0; i < 4; i++) ov[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
                *reinterpret_cast<uint4 *>(a.out + (size_t)p * COUT + n0) = o;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 2) tmem_free(tmem, TCOLS);
}

// k_conv_rows: the 3x3 convolution for 16, 32 or 64 input channels, persistent,
// on 2-D tiles of MT image rows x 128 columns of the padded grid.  The
// activation is staged as one 3-D TMA box of all CIN channels x 130 columns
// x (MT + 2) rows (the tile with a one-pixel halo): pixel rows of 32, 64 or
// 128 bytes with the matching swizzle, so that
//   * the operand of output row mt at tap (dy, dx) is the box's pixel
//     (mt + dy) * 130 + dx onwards -- a whole number of pixel rows added to
//     the descriptor's start address (base offset 0): the TMA writes and the
//     MMA reads apply the swizzle to the absolute shared-memory address, so
//     a start part-way into the pattern reads the rows as they were written
//     (the same holds for the 32-byte K offsets within a swizzled row);
//   * the three tap rows of neighbouring output rows share staged rows, so a
//     tile stages (MT + 2) / (3 MT) of what one box per tap row would.
// Each CTA walks the tiles with stride gridDim.x:
//   warp 0 lane 0  TMA producer: one stage per tile through a ring of
//                  ROWS_RING slots;
//   warp 1 lane 0  MMA issuer into one of two tensor-memory accumulators
//                  (tile parity), so a tile's epilogue overlaps the next
//                  tile's loads and MMAs;
//   warps 2..9     epilogue: warp w reads tensor-memory lanes 32*(w%4)..
//                  of every other output row (two warps per lane quarter).
// The nine taps' weights are staged once per CTA.  Every wait is bounded;
// a wait that gives up sets ST_UNET_TIMEOUT and a shared abort flag that
// ends every role's loop, after which the producer waits (bounded) for its
// copies still in flight and the MMA issuer for its MMAs before the tensor
// memory is freed.
template <int CIN, int COUT>
__host__ __device__ constexpr int conv_rows_mt() {
    return CIN == 16 ? 4 : (CIN == 32 ? 4 : 2);
}
static constexpr int ROWS_BOXW = 130;      // staged columns: 128 outputs and a halo column each side
static constexpr int ROWS_RING = 2;        // tile stages in flight (default)
static constexpr int ROWS_THREADS = 320;   // producer, MMA, eight epilogue warps
static constexpr int ROWS_EPI_WARPS = 8;

template <int CIN, int COUT>
struct RowsCfg {
    static constexpr int MT = conv_rows_mt<CIN, COUT>();
    static constexpr int ROWB = CIN * 2;                                // bytes per staged pixel (= swizzle span)
    static constexpr int BOXB = ROWB * ROWS_BOXW * (MT + 2);            // the tile's box
    static constexpr int ASLOT = (BOXB + 1023) / 1024 * 1024;           // one tile
    static constexpr int BT = (COUT * CIN * 2 + 1023) / 1024 * 1024;    // one tap's weights
    static constexpr int RING = CIN == 16 ? 4 : ROWS_RING;              // tile stages in flight (measured)
    static constexpr int NC = MT * COUT;                                // columns per accumulator
    static constexpr uint32_t TCOLS = 2 * NC <= 32 ? 32 : (2 * NC <= 64 ? 64 : (2 * NC <= 128 ? 128 : (2 * NC <= 256 ? 256 : 512)));
    static constexpr unsigned ATX = BOXB;
    static constexpr unsigned BTX = 9 * COUT * CIN * 2;
    static constexpr size_t SMEM = 9 * (size_t)BT + RING * (size_t)ASLOT + 1024;
    static_assert(CIN == 16 || CIN == 32 || CIN == 64, "pixel rows of 32, 64 or 128 bytes");
    static_assert(MT % 2 == 0, "two epilogue warps per lane quarter take alternate rows");
    static_assert(2 * NC <= 512, "layout");
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(ROWS_THREADS) k_conv_rows(const __grid_constant__ CUtensorMap ta,
                                                            const __grid_constant__ CUtensorMap tb,
                                                            ConvArgs a) {
    using R = RowsCfg<CIN, COUT>;
    constexpr int MT = R::MT;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[R::RING], empty[R::RING], tfull[2], tempty[2], wfull, done;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_;
    __shared__ float sbias[COUT];
    constexpr int RB = COUT <= 16 ? 2 : 1;   // output rows per tensor-memory wait in the epilogue
    static_assert((MT / 2) % RB == 0, "each epilogue warp's rows come in whole batches");
    unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    unsigned char *sw = smem, *ring = smem + 9 * R::BT;
    // the bias is a parameter of the layer: no kernel the forward pass
    // overlaps with writes it
    for (int i = threadIdx.x; i < COUT; i += blockDim.x) sbias[i] = a.bias ? a.bias[i] : 0.f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int HP = a.H + 2;                               // padded rows
    const int ncb = cdiv_dev(a.Wp, 128), ntiles = cdiv_dev(HP, MT) * ncb;

    if (threadIdx.x == 0) {
        for (int s = 0; s < R::RING; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], ROWS_EPI_WARPS);
        }
        mbar_init(&wfull, 1);
        mbar_init(&done, 1);
        abort_ = 0;
    }
    if (warp == 1) tmem_alloc(&tmem_base, R::TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    pdl_trigger();
    pdl_wait();          // the set-up above overlapped the previous kernel's tail

    if (warp == 0 && lane == 0) {
        mbar_expect_tx(&wfull, R::BTX);
        for (int t = 0; t < 9; t++) tma_load_2d(sw + t * R::BT, &tb, 0, (a.tap_reverse ? 8 - t : t) * COUT, &wfull);
        int s = 0;
        for (int tile = blockIdx.x; tile < ntiles && !abort_; tile += gridDim.x, s++) {
            const int r0 = (tile / ncb) * MT, c0 = (tile % ncb) * 128;
            const int slot = s % R::RING;
            if (s >= R::RING && !mbar_wait(&empty[slot], ((s / R::RING) - 1) & 1)) {
                atomicOr(a.status, ST_UNET_TIMEOUT);
                abort_ = 1;
                break;
            }
            unsigned char *sa = ring + slot * R::ASLOT;
            mbar_expect_tx(&full[slot], R::ATX);
            tma_load_3d(sa, &ta, 0, c0 - 1, r0 - 1, &full[slot]);
        }
        // the copies of the last ring round have landed before the CTA exits
        for (int q = s - R::RING < 0 ? 0 : s - R::RING; q < s; q++)
            if (!mbar_wait(&full[q % R::RING], (q / R::RING) & 1)) atomicOr(a.status, ST_UNET_TIMEOUT);
        if (!mbar_wait(&wfull, 0)) atomicOr(a.status, ST_UNET_TIMEOUT);
    } else if (warp == 1 && lane == 0) {
        constexpr uint32_t idesc = idesc_bf16_f32(COUT);
        const uint32_t sb = smem_u32(sw), sring = smem_u32(ring);
        bool ok = mbar_wait(&wfull, 0);
        int li = 0;
        for (int tile = blockIdx.x; ok && tile < ntiles && !abort_; tile += gridDim.x, li++) {
            const int buf = li & 1, slot = li % R::RING;
            if (li >= 2 && !mbar_wait(&tempty[buf], ((li >> 1) - 1) & 1)) { ok = false; break; }
            if (!mbar_wait(&full[slot], (li / R::RING) & 1)) { ok = false; break; }
            tc_fence_after();
            const uint32_t acc = tmem + (uint32_t)(buf * R::NC), sa = sring + slot * R::ASLOT;
#pragma unroll
            for (int dy = 0; dy < 3; dy++)
#pragma unroll
                for (int dx = 0; dx < 3; dx++)
#pragma unroll
                    for (int mt = 0; mt < MT; mt++)
#pragma unroll
                        for (int ks = 0; ks < CIN / 16; ks++)
                            mma_bf16(acc + (uint32_t)(mt * COUT),
                                     smem_desc(sa + ((mt + dy) * ROWS_BOXW + dx) * R::ROWB + 32 * ks, R::ROWB),
                                     smem_desc(sb + (3 * dy + dx) * R::BT + 32 * ks, CIN * 2), idesc,
                                     (dy > 0 || dx > 0 || ks > 0) ? 1u : 0u);
            mma_commit(&empty[slot]);
            mma_commit(&tfull[buf]);
        }
        if (!ok) {
            atomicOr(a.status, ST_UNET_TIMEOUT);
            abort_ = 1;
        }
        // every MMA this thread issued has completed before the memory is freed
        mma_commit(&done);
        if (!mbar_wait(&done, 0)) atomicOr(a.status, ST_UNET_TIMEOUT);
    } else if (warp >= 2) {
        const int q = warp & 3;                     // tensor-memory lane quarter of this warp
        const int half = (warp - 2) >> 2;           // output rows half, half + 2, ...
        int li = 0;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, li++) {
            const int buf = li & 1;
            const bool ok = !abort_ && mbar_wait(&tfull[buf], (li >> 1) & 1);
            if (!ok) {
                if (lane == 0 && !abort_) {
                    atomicOr(a.status, ST_UNET_TIMEOUT);
                    abort_ = 1;
                }
                break;
            }
            tc_fence_after();
            const int r0 = (tile / ncb) * MT, col = (tile % ncb) * 128 + 32 * q + lane;
            // RB of this warp's output rows (half, half + 2, ...) per tensor-memory wait
#pragma unroll 1
            for (int m0 = half; m0 < MT; m0 += 2 * RB) {
                uint32_t r[RB][COUT];
#pragma unroll
                for (int j = 0; j < RB; j++)
#pragma unroll
                    for (int n0 = 0; n0 < COUT; n0 += 8)
                        tmem_ld8_issue(tmem + ((uint32_t)(32 * q) << 16) +
                                           (uint32_t)(buf * R::NC + (m0 + 2 * j) * COUT + n0),
                                       r[j] + n0);
#pragma unroll
                for (int j = 0; j < RB; j++)
#pragma unroll
                    for (int n0 = 0; n0 < COUT; n0 += 8) tmem_ld_wait(r[j] + n0);
#pragma unroll
                for (int j = 0; j < RB; j++) {
                    const int row = r0 + m0 + 2 * j;
                    if (!(row < HP && col < a.Wp)) continue;
                    const bool in = row >= 1 && row <= a.H && col >= 1 && col <= a.W;
                    const size_t p = (size_t)row * a.Wp + col;
#pragma unroll
                    for (int n0 = 0; n0 < COUT; n0 += 8) {
                        float v[8];
#pragma unroll
                        for (int i = 0; i < 8; i++) {
                            float x = __uint_as_float(r[j][n0 + i]) + sbias[n0 + i];
                            if (a.relu) x = fmaxf(x, 0.f);
                            v[i] = (in ? x : 0.f);
                        }
                        if (a.mask && in) {
                            const uint4 mk = *reinterpret_cast<const uint4 *>(a.mask + p * COUT + n0);
                            const __nv_bfloat16 *mv = reinterpret_cast<const __nv_bfloat16 *>(&mk);
#pragma unroll
                            for (int i = 0; i < 8; i++)
                                if (!(__bfloat162float(mv[i]) > 0.f)) v[i] = 0.f;
                        }
                        if (a.out_f32) {
                            if (n0 == 0) a.out_f32[p] = v[0];
                        } else {
                            uint4 o;
                            __nv_bfloat162 *ov = reinterpret_cast<__nv_bfloat162 *>(&o);
#pragma unroll
                            for (int i = 0; i < 4; i++) ov[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
                            *reinterpret_cast<uint4 *>(a.out + p * COUT + n0) = o;
                        }
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[buf]);
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    if (warp == 1) tmem_free(tmem, R::TCOLS);
}

struct WgradArgs {
    int Cin, Cout, Wp, P;
    int chunk;                // pixels per CTA (a multiple of 64)
    float *part;              // [chunks][9][Cout][Cin] FP32 partial products
    unsigned *status;
};

// B operands: X pre-shifted by dx = -1, 0, +1 (planar, Cin rows of P pixels)
struct WgradMaps {
    CUtensorMap dy;           // planar dY: Cout rows of P pixels, box 64 x 128
    CUtensorMap x[3];         // planar X shifted by dx, box 64 x Cin
};

template <int CIN>
__global__ void __launch_bounds__(CONV_THREADS) k_conv_wgrad(const __grid_constant__ WgradMaps maps,
                                                             WgradArgs a) {
    constexpr int ROWB = 128;                            // 64 pixels of BF16
    constexpr int ABYTES = 128 * ROWB, BBYTES = CIN * ROWB;
    constexpr int STAGE = ((ABYTES + BBYTES) + 1023) / 1024 * 1024;
    constexpr uint32_t TCOLS = CIN <= 32 ? 32 : (CIN <= 64 ? 64 : (CIN <= 128 ? 128 : 256));
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[CONV_STAGES], empty[CONV_STAGES], done;
    __shared__ uint32_t tmem_base;
    unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.y, dy = t / 3 - 1, dx = t % 3 - 1;
    const int p0 = blockIdx.x * a.chunk;
    const int nsteps = min(a.chunk, a.P - p0 + 63) / 64;

    if (threadIdx.x == 0) {
        for (int s = 0; s < CONV_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&done, 1);
    }
    if (warp == 2) tmem_alloc(&tmem_base, TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == 0 && lane == 0) {
        for (int s = 0; s < nsteps; s++) {
            const int st = s % CONV_STAGES;
            if (s >= CONV_STAGES && !mbar_wait(&empty[st], ((s / CONV_STAGES) - 1) & 1)) {
                atomicOr(a.status, ST_UNET_TIMEOUT);
                break;
            }
            unsigned char *sa = smem + st * STAGE, *sb = sa + ABYTES;
            const int px = p0 + 64 * s;
            mbar_expect_tx(&full[st], ABYTES + BBYTES);
            tma_load_2d(sa, &maps.dy, px, 0, &full[st]);
            tma_load_2d(sb, &maps.x[dx + 1], px + dy * a.Wp, 0, &full[st]);
        }
    } else if (warp == 1 && lane == 0) {
        constexpr uint32_t idesc = idesc_bf16_f32(CIN);
        for (int s = 0; s < nsteps; s++) {
            const int st = s % CONV_STAGES;
            if (!mbar_wait(&full[st], (s / CONV_STAGES) & 1)) {
                atomicOr(a.status, ST_UNET_TIMEOUT);
                break;
            }
            tc_fence_after();
            const uint32_t sa = smem_u32(smem + st * STAGE), sb = sa + ABYTES;
#pragma unroll
            for (int k = 0; k < 4; k++)
                mma_bf16(tmem, smem_desc(sa + 32 * k, ROWB), smem_desc(sb + 32 * k, ROWB), idesc,
                         (s > 0 || k > 0) ? 1u : 0u);
            mma_commit(&empty[st]);
        }
        mma_commit(&done);
    }
    __syncwarp();
    const bool ok = mbar_wait(&done, 0) && nsteps > 0;
    if (!ok && nsteps > 0 && threadIdx.x == 0) atomicOr(a.status, ST_UNET_TIMEOUT);
    tc_fence_after();
    const int co = 32 * warp + lane;
#pragma unroll
    for (int n0 = 0; n0 < CIN; n0 += 8) {
        float v[8];
        tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)n0, v);
        if (co >= a.Cout) continue;
        float4 *dst = reinterpret_cast<float4 *>(a.part + (((size_t)blockIdx.x * 9 + t) * a.Cout + co) * a.Cin + n0);
        dst[0] = ok ? make_float4(v[0], v[1], v[2], v[3]) : make_float4(0.f, 0.f, 0.f, 0.f);
        dst[1] = ok ? make_float4(v[4], v[5], v[6], v[7]) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 2) tmem_free(tmem, TCOLS);
}

// out[i] = sum over k < nparts of part[k * n + i], in order of k
__global__ void k_sum_parts(const float *__restrict__ part, int nparts, int n, float *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.f;
    for (int k = 0; k < nparts; k++) s += part[(size_t)k * n + i];
    out[i] = s;
}

}  // namespace qd
