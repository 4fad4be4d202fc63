// qdeq_internal.cuh -- shared definitions of the GB300 hot-path library.
//
// Device data layout (one solver, one GPU):
//   level l of the multigrid hierarchy holds N x K nodes (N rows along the
//   fault = depth, K columns off-fault), row-major with a row pitch P that
//   is a multiple of 32 elements, so every row starts on a 256-byte
//   boundary.  Face moduli are repacked from the reference's staggered
//   mu_equi into three dense arrays per level:
//     cx[j*P + k]   face between (j,k) and (j,k+1),   k = 0..K-2
//     cz[j*P + k]   face between (j-1,k) and (j,k),   j = 0..N (N+1 rows)
//     dinv[j*P + k] 1 / (cx[k-1] + cx[k] + cz[j] + cz[j+1])
//   The reference's row quirks are folded into cz (see mg.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/qdeq.h"

#define QD_MAXLEV 16

namespace qd {

void set_error(const char *fmt, ...);

#define QD_CUDA(call)                                                              \
    do {                                                                           \
        cudaError_t e__ = (call);                                                  \
        if (e__ != cudaSuccess) {                                                  \
            (void)cudaGetLastError(); /* clear a non-sticky error for later calls */ \
            ::qd::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call,            \
                            cudaGetErrorString(e__));                              \
            return QD_ERR_CUDA;                                                    \
        }                                                                          \
    } while (0)

#define QD_LAUNCH_CHECK(s)                                                         \
    do {                                                                           \
        (s)->launches++;                                                           \
        cudaError_t e__ = cudaPeekAtLastError();                                   \
        if (e__ != cudaSuccess) {                                                  \
            ::qd::set_error("%s:%d: launch: %s", __FILE__, __LINE__,               \
                            cudaGetErrorString(e__));                              \
            return QD_ERR_CUDA;                                                    \
        }                                                                          \
    } while (0)

#define QD_TRY(expr)                                                               \
    do {                                                                           \
        int rc__ = (expr);                                                         \
        if (rc__ != QD_OK) return rc__;                                            \
    } while (0)

template <typename T>
struct Level {
    T *u = nullptr;      // level 0: the solution u; coarse: the error e
    T *f = nullptr;      // right-hand side (nullptr: identically zero)
    T *r = nullptr;      // residual scratch
    T *cx = nullptr, *cz = nullptr, *dinv = nullptr;
    T *diag = nullptr;   // level 0 of the FP64 hierarchy only: cx[k-1]+cx[k]+cz[j]+cz[j+1]
};

struct LevelDims {
    int N, K, P;
    double h2, inv_h2;
};

// Device-side fault / RK43 state (nz-long vectors, entries 1..nk used).
struct FaultState {
    double *mu0 = nullptr;  // node modulus at the fault column (fault.cpp:153)
    double *a = nullptr, *b = nullptr, *eta = nullptr, *Tn0 = nullptr;
    double *tau0 = nullptr, *SlipShift = nullptr;
    double *Slip = nullptr, *psi = nullptr, *Ts = nullptr, *Tn = nullptr;
    double *kslip[7] = {}, *kpsi[7] = {}, *fV[7] = {}, *fdpsi[7] = {};
    double *y3s = nullptr, *y3p = nullptr, *y4s = nullptr, *y4p = nullptr;
    int *iters = nullptr;
    double f0 = 0, V0 = 0, L = 0, Vini = 0;
    int have_tau0 = 0;
};

// Status word written by device kernels (bit flags + first bad node).
struct DevStatus {
    unsigned int flags;
    int bad_node;
};
enum : unsigned int { ST_NEWTON_NAN = 1u, ST_NEWTON_CAP = 2u, ST_NEWTON_BRACKET = 4u };
// set by a multigrid tile kernel whose TMA staging did not complete
static constexpr unsigned int ST_TMA_TIMEOUT = 8u;

// The learned correction's default cost in V-cycles for the measured gate:
// one inference on the level-1 grid of a 1025^2 solver (181 us) against one
// V-cycle there with its level-0 residual (about 100 us) is about two cycles.
static constexpr double kNetCostCycles = 2.0;

// state of the device-driven multigrid loop (mg_graph.cu)
struct SolveState {
    double thr, delta, r0;
    int cycles;                           // V-cycles of the last solve
    int flag;                             // 1: non-finite norm, 2: cycle cap (sticky)
    int go;                               // the last "run another cycle" decision
    unsigned long long total_cycles, total_solves;
    unsigned long long kernels;           // kernels the solve graphs ran
    int net;                              // the network corrected the last solve's guess
    unsigned long long net_solves;        // solves whose guess the network corrected
    double log_rho;                       // running mean of log(||r|| after / before a V-cycle)
    unsigned long long rho_samples;       // cycles in that mean
    // the corrected solves' V-cycles: those their guesses needed (estimated
    // from the measured reduction per cycle) and those they took
    double net_cycles_needed, net_cycles_taken;
    // the most V-cycles any solve's first guess needed since the host last
    // cleared it (1e30 while no cycle has been measured): the host's
    // warm-start standby reads it once per RK attempt
    double need_max;
    // the next correction is a level-0 smoothing pass instead of a V-cycle
    // (set by the check after a V-cycle that left ||r|| within the solver's
    // smoothing ratio of the threshold), and how many such passes ran
    int smooth;
    unsigned long long total_smooths;
};

// ---- programmatic dependent launch ----------------------------------------
// A kernel launched with programmatic stream serialization (launch_pdl) may
// be scheduled while the kernel before it drains, which hides the launch
// latency between dependent kernels.  Such a kernel calls pdl_trigger (let
// the next kernel start launching) and pdl_wait (block until the previous
// kernel has completed and its memory operations are visible) before it
// touches anything the previous kernel produced or reads.  Both are no-ops
// in a kernel launched without the attribute.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
static inline cudaError_t launch_pdl(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                     cudaStream_t st, Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<Args &&>(args)...);
}

// The solve loop's decisions, shared by the stand-alone decision kernels and
// the reductions that fuse them: after the prologue's norms (scal[0] =
// ||r||^2 of the guess, scal[1] = ||r0||^2 for the relative tolerance) and
// after each cycle.  Both return "run another cycle"; the caller sets the
// graph's loop condition from it.
// phase 0: a solve's only first decision; 1: the first decision of a solve
// whose guess the network corrects when ||r|| of the guess exceeds
// ratio x the threshold (st->net): net_ratio >= 1 that fixed ratio;
// net_ratio <= 0 the measured rule, ratio rho^-(1 + c) with c = -net_ratio
// the network's cost in V-cycles and rho = exp(log_rho) the measured
// reduction per cycle -- the guess would need more than 1 + c cycles
// (ratio 1 while no cycle has been measured); 2: the decision after that
// correction (the same solve)
// V-cycles that take ||r|| = delta below thr at the mean reduction
// exp(log_rho) < 1 per cycle (an estimate, in binary32)
__device__ inline double cycles_needed(double delta, double thr, double log_rho) {
    return (double)ceilf(logf((float)delta / (float)thr) / -(float)log_rho);
}

// delta = ||r|| of the guess, r0 = ||r0|| (read with the relative
// tolerance only)
__device__ inline int solve_begin_dev(double delta, double r0, SolveState *st, int rel, double tol, int n_kernels,
                                      int phase, double net_ratio = 1.0, int n_kernels_gated = 0) {
    if (!rel) r0 = 0.0;
    const double thr = rel ? (r0 > 0.0 ? tol * r0 : tol) : tol;
    st->r0 = r0;
    st->thr = thr;
    st->delta = delta;
    st->cycles = 0;
    st->smooth = 0;
    if (phase == 2) st->net_solves++;
    else st->total_solves++;
    st->kernels += (unsigned long long)n_kernels;
    int go = !(delta <= thr);
    // a non-finite norm of the guess or of the zero-interior residual (the
    // relative tolerance's scale): the boundary data or the guess hold an
    // infinity or a NaN, and no cycle can reach the tolerance
    if (!isfinite(delta) || !isfinite(thr)) {
        st->flag |= 1;
        go = 0;
    }
    st->go = go;
    if (!go) st->kernels += (unsigned long long)n_kernels_gated;
    // the estimates below (cycles a guess needs, the network's gate) take
    // their logarithms and exponentials in binary32: one thread's chain of
    // FP64 transcendentals is microseconds on GB300's FP64 pipe
    if (go && phase != 2) {
        const double need = (st->rho_samples && st->log_rho < 0.0) ? cycles_needed(delta, thr, st->log_rho) : 1e30;
        st->need_max = fmax(st->need_max, need);
    }
    if (phase == 0) st->net = 0;
    else if (phase == 1) {
        const double ratio =
            net_ratio > 0.0 ? net_ratio
                            : (st->rho_samples ? (double)expf(-(float)((1.0 - net_ratio) * st->log_rho)) : 1.0);
        st->net = go && !(delta <= ratio * thr);
        if (st->net && st->rho_samples && st->log_rho < 0.0)
            st->net_cycles_needed += cycles_needed(delta, thr, st->log_rho);
    }
    return go;
}

// After a correction: the running reduction per V-cycle (V-cycles only),
// the loop's next decision and, with smooth_ratio > 1 (mixed precision),
// whether the next correction is a level-0 smoothing pass: once per solve,
// after a V-cycle that left ||r|| within smooth_ratio of the threshold
// (there the residual is mostly the rough part a smoothing pass removes;
// measured at 1025^2: one pass of four sweeps cuts ||r|| to about 1/3).
// cycles counts both kinds against the cap; n_kernels and n_kernels_smooth
// are the kernels of the two kinds of iteration.
__device__ inline int solve_check_dev(double delta, SolveState *st, int max_cycles, int n_kernels,
                                      double smooth_ratio = 0.0, int n_kernels_smooth = 0) {
    const bool was_smooth = st->smooth != 0;
    // the cycle's reduction factor, into the running mean of its log
    // (weight 1/8 after the first eight; factors clamped to [1e-6, 1])
    const float red = (float)delta / (float)st->delta;   // an estimate: binary32
    if (!was_smooth && st->delta > 0.0 && isfinite(red)) {
        const double l = (double)logf(fminf(fmaxf(red, 1e-6f), 1.0f));
        const double w = st->rho_samples < 8 ? 1.0 / (double)(st->rho_samples + 1) : 0.125;
        st->log_rho += w * (l - st->log_rho);
        st->rho_samples++;
    }
    st->delta = delta;
    st->cycles++;
    if (was_smooth) {
        st->total_smooths++;
        st->kernels += (unsigned long long)n_kernels_smooth;
    } else {
        st->total_cycles++;
        st->kernels += (unsigned long long)n_kernels;
    }
    int go = !(delta <= st->thr);
    if (go && !isfinite(delta)) {
        st->flag |= 1;
        go = 0;
    }
    if (go && max_cycles > 0 && st->cycles >= max_cycles) {
        st->flag |= 2;
        go = 0;
    }
    if (!go && st->net) st->net_cycles_taken += st->cycles;
    st->smooth = go && !was_smooth && smooth_ratio > 1.0 && delta <= smooth_ratio * st->thr;
    st->go = go;
    return go;
}

// a decision fused into the last block of the level-0 residual's
// reduction (mixed precision): mode 1 also computes ||r0||^2 and takes the
// first decision (phase as for solve_begin_dev; phase 1 also sets h_net to
// the decision), mode 2 the decision after a cycle; mode 0 none
struct Decide {
    int mode, rel, max_cycles, n_kernels, in_graph, phase;
    double tol, net_ratio;
    cudaGraphConditionalHandle h, h_net;
    SolveState *st;
    // mode 2: the level-0 smoothing pass (smooth_ratio > 1: enabled; its
    // condition goes to h_smooth in a graph; n_kernels_smooth as n_kernels)
    double smooth_ratio;
    int n_kernels_smooth;
    cudaGraphConditionalHandle h_smooth;
    // mode 2: non-null, the check is skipped when *gate is 0 (the graph's
    // first V-cycle, after a prologue that found the guess converged);
    // mode 1: the kernels so skipped, counted as launched
    const int *gate;
    int n_kernels_gated;
};

// binary64 -> binary32 with round-to-nearest-even, on the integer pipes.
// GB300's FP64 pipe, which issues about one instruction per SM clock, also
// executes the hardware F2F conversion; this routine follows the IEEE
// 754 definition directly: keep the top 23 of the 52 fraction bits, round on
// the 29 dropped bits (ties to even) and let a carry out of the fraction
// bump the exponent (which also rounds the largest values to infinity as
// RNE requires).  Results below the normal binary32 range round the full
// 53-bit significand to a multiple of 2^-149 the same way (a carry reaches
// the smallest normal); |x| >= 2^128 gives infinity; NaN stays NaN.  No
// FP64 instruction is involved.
__device__ __forceinline__ float d2f_rne(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), sign = hi & 0x80000000u;
    const int ex = (int)((hi >> 20) & 0x7FFu);
    const unsigned long long frac = b & 0xFFFFFFFFFFFFFull;
    if (ex == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (frac ? 0x00400000u : 0u));
    const int e = ex - 1023 + 127;
    if (e >= 255) return __uint_as_float(sign | 0x7F800000u);
    if (e >= 1) {
        unsigned q = (unsigned)(frac >> 29);
        const unsigned rem = (unsigned)(frac & 0x1FFFFFFFull), half = 0x10000000u;
        q += (rem > half || (rem == half && (q & 1u))) ? 1u : 0u;
        return __uint_as_float((sign | ((unsigned)e << 23)) + q);
    }
    // binary32 subnormal range: units of 2^-149 are m >> (30 - e)
    const int shift = 30 - e;
    if (ex == 0 || shift >= 54) return __uint_as_float(sign);
    const unsigned long long m = frac | (1ull << 52);
    const unsigned long long rem = m & ((1ull << shift) - 1), half = 1ull << (shift - 1);
    unsigned q = (unsigned)(m >> shift);
    q += (rem > half || (rem == half && (q & 1u))) ? 1u : 0u;
    return __uint_as_float(sign | q);
}

// binary64 x -> a pair of binary32 (hi, lo) with x = hi + lo to within
// 2^-48 |x| (the double-float representation of Dekker, "A floating-point
// technique for extending the available precision", 1971), in about 16
// integer and FP32 instructions (GB300's FP64 pipe, which executes the
// hardware conversion, issues about one instruction per SM clock).  With x =
// +-1.f 2^(e-1023): hi keeps the sign, the exponent and the top 23 of the 52
// fraction bits (truncated), built from the high word rebiased and the top
// three bits of the low word; the 29 bits below are an integer m, and lo =
// m 2^(e-1075) is m converted to binary32 (rounded to 24 bits) times that
// power of two, exact; |lo| < ulp(hi).  |x| < 2^-74 (zeros included) gives
// (+-0, 0): an absolute error under 2^-74, far below any displacement the
// solver resolves; |x| >= 2^128 gives (+-inf, 0); NaN gives (NaN, 0).
__device__ __forceinline__ float2 d_split(double x) {
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned sign = hw & 0x80000000u, mag = hw & 0x7FFFFFFFu;   // exponent and top 20 fraction bits
    if (mag < (949u << 20)) return make_float2(__uint_as_float(sign), 0.f);
    if (mag >= (1151u << 20)) {
        const bool nan = mag > 0x7FF00000u || (mag == 0x7FF00000u && lw != 0u);
        return make_float2(__uint_as_float(sign | 0x7F800000u | (nan ? 0x00400000u : 0u)), 0.f);
    }
    const float hi = __uint_as_float(sign | ((mag - (896u << 20)) << 3) | (lw >> 29));
    const float scale = __uint_as_float(sign | (((mag >> 20) - 948u) << 23));   // +-2^(e-1075)
    return make_float2(hi, __uint2float_rn(lw & 0x1FFFFFFFu) * scale);
}

// s + lo += (ch + cl)(uh + ul): the hi product exactly (p + e) into the
// running sum by two-sum, everything smaller into lo.  The _rn intrinsics
// keep the compiler from contracting the product into the sum.
// s + lo = (ch + cl)(uh + ul): the first term of a df_acc sum
__device__ __forceinline__ void df_first(float ch, float cl, float uh, float ul, float &s, float &lo) {
    s = __fmul_rn(ch, uh);
    lo = fmaf(ch, ul, fmaf(cl, uh, fmaf(ch, uh, -s)));
}

__device__ __forceinline__ void df_acc(float ch, float cl, float uh, float ul, float &s, float &lo) {
    const float p = __fmul_rn(ch, uh);
    const float e = fmaf(ch, uh, -p);
    const float t = fmaf(ch, ul, fmaf(cl, uh, e));
    const float sn = __fadd_rn(s, p);
    const float bb = __fsub_rn(sn, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(sn, bb)), __fsub_rn(p, bb));
    s = sn;
    lo = __fadd_rn(lo, __fadd_rn(err, t));
}

// binary32 -> binary64 exactly, on the integer pipes (GB300's FP64 pipe
// executes the hardware conversion): sign, exponent rebiased by 1023 - 127,
// the 23 fraction bits at the top of the 52.  Subnormal inputs give +-0: in
// the double-float sums here they can only be rounding debris far below the
// values' resolution.  Infinities and NaN carry over.
__device__ __forceinline__ double f2d_exact(float x) {
    const unsigned b = __float_as_uint(x), sign = b & 0x80000000u, e = (b >> 23) & 0xFFu, m = b & 0x7FFFFFu;
    if (e == 0u) return __hiloint2double((int)sign, 0);
    const unsigned ex = e == 0xFFu ? 0x7FFu : e + (1023u - 127u);
    return __hiloint2double((int)(sign | (ex << 20) | (m >> 3)), (int)(m << 29));
}

// x as a double-float pair hi + lo (hi = x rounded to binary32, lo = the
// rest rounded to binary32: x to about 2^-48 of itself within binary32's
// range), without the FP64 pipe's conversion
__device__ __forceinline__ float2 df_of(double x) {
    const float hi = d2f_rne(x);
    return make_float2(hi, d2f_rne(x - f2d_exact(hi)));
}

// a + b for double-float pairs: Knuth's two-sum of the high parts, the low
// parts and the rounding error summed, then renormalised (about 2^-44 of
// the sum for sums of like-signed terms)
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float s = __fadd_rn(a.x, b.x);
    const float bb = __fsub_rn(s, a.x);
    const float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
    const float t = __fadd_rn(e, __fadd_rn(a.y, b.y));
    const float hi = __fadd_rn(s, t);
    return make_float2(hi, __fsub_rn(t, __fsub_rn(hi, s)));
}

// 1/sqrt(x) in FP64 from a binary32 reciprocal square root and one Newton
// step r (3 - x r^2) / 2: within about 1e-14 of itself, four dependent FP64
// instructions; outside binary32's range, and for 0, negative or
// non-finite x, the library's rsqrt
__device__ __forceinline__ double rsqrt_refined(double x) {
    const float xf = d2f_rne(x);
    if (!(xf > 0.f) || isinf(xf) || !isfinite(x)) return rsqrt(x);
    const double r = f2d_exact(rsqrtf(xf));
    return r * fma(-0.5 * x * r, r, 1.5);
}

// a / b in FP64 from a binary32 reciprocal and two Newton corrections
// (the reciprocal's, then the quotient's): within about an ulp of a / b in
// five dependent FP64 instructions; where b is 0, not finite or outside
// binary32's range, the library's division
__device__ __forceinline__ double div_refined(double a, double b) {
    const float bf = d2f_rne(b);
    if (!(fabsf(bf) > 0.f) || isinf(bf) || !isfinite(b)) return a / b;
    double r = f2d_exact(__frcp_rn(bf));
    r = fma(r, fma(-b, r, 1.0), r);
    const double q = a * r;
    return fma(r, fma(-b, q, a), q);
}

// e^d for |d| <= 1e-3 by its Taylor series to d^6 (error below 2e-25)
__device__ __forceinline__ double exp_small(double d) {
    return 1.0 + d * (1.0 + d * (1.0 / 2.0 + d * (1.0 / 6.0 + d * (1.0 / 24.0 + d * (1.0 / 120.0 + d * (1.0 / 720.0))))));
}

// sqrt(x) in FP64 from a binary32 reciprocal square root and one Newton
// step (Heron's correction y + (x - y^2) r / 2): within a few units of
// 2^-52 of sqrt(x), with a shorter chain of dependent FP64 instructions
// than the library's sqrt; outside binary32's range, and for 0, negative
// or non-finite x, the library's sqrt
__device__ __forceinline__ double sqrt_refined(double x) {
    const float xf = d2f_rne(x);
    if (!(xf > 0.f) || isinf(xf) || !isfinite(x)) return sqrt(x);
    const double r = f2d_exact(rsqrtf(xf));
    const double y = x * r;
    return fma(0.5 * r, fma(-y, y, x), y);
}

}  // namespace qd

struct qd_solver {
    int ni, nk, nx, nz;
    double dh;
    qd_mg_options opt;
    int nlev;
    int n_sm;              // the device's SM count
    qd::LevelDims dims[QD_MAXLEV];
    qd::Level<double> L64[QD_MAXLEV];
    qd::Level<float> L32[QD_MAXLEV];
    cudaStream_t stream;
    double *d_partial;     // per-block reduction partials
    unsigned *d_count;     // blocks done, for reductions finished by their last block
    // level-0 cx, cz and diag as double-float pairs (d_split), for the
    // mixed-precision residual; null in FP64 solvers
    float2 *res_cx, *res_cz, *res_dg;
    double *d_ainv64;      // dense inverse of the coarsest-level operator (or null)
    float *d_ainv32;
    int n_cint;            // its order: coarsest N * (K-2) interior unknowns
    void *tma_cache;       // tensor maps of the tile kernels (mg_fused.cu)
    void *d_tail_img[2];   // coarse-tail coefficient images, FP32 [0] and FP64 [1]
    void *unet;            // attached warm-start network (unet.cu), or null
    bool net_paused;       // solves leave the attached network out (the autotuner's timing)
    bool net_standby;      // ... and while no guess of the last RK attempt needed the network
    double net_ratio;      // the network's gate: >= 1 a fixed ratio of ||r|| to the threshold;
                           // <= 0 the measured rule with a cost of -net_ratio V-cycles
    double net_cost;       // the measured rule's cost (V-cycles)
    int newton_start;      // the Newton solve's start: 0 the reference's x = 0, 1 a binary32 solve
    void *history;         // ring of earlier solutions for the initial guess (history.cu), or null
    void *snapshot;        // the snapshot writer in flight (io.cu), or null
    // staging of the host transfers (allocated on first use): the ghosted
    // nz x nx field and five nz-vectors on the device, five nz-vectors pinned
    double *io_dev, *io_host;
    int tail_l0;           // first level of the coarse tail
    int tail_sweeps;       // pre- and post-sweeps on the tail's levels (0: the fine levels' nu_pre, nu_post)
    double smooth_ratio;   // mixed precision: a level-0 smoothing pass instead of a second V-cycle
                           // within this ratio of the threshold (0: off)
    const int *cycle_gate; // while capturing a solve graph's first V-cycle: the device flag
                           // (SolveState.go) its kernels check to skip themselves; else null
    int box_up, box_down;  // staged tile box widths of k_up / k_down (0: the defaults)
    void *solve_graph;     // the instantiated multigrid graph (mg_graph.cu)
    qd::SolveState *d_solve, *h_solve;
    // device addresses of the pinned h_scal, h_solve and h_status (null when
    // the device cannot address them): the error kernel's attempt report
    double *dh_scal;
    qd::SolveState *dh_solve;
    qd::DevStatus *dh_status;
    int n_partial;
    double *d_scal;        // device scalars: [0] ||r||^2, [1] ||r0||^2, [2] totErr, [3] the step of mr_step
    double *h_scal;        // pinned mirror
    qd::DevStatus *d_status;
    qd::DevStatus *h_status;
    qd::FaultState F;
    int fault_ready;
    // RK43 state (PARAMS)
    qd_rk43_params P;
    double t, dt, errA[2];
    int it;
    int started;
    // counters
    long long solves, vcycles, attempts, steps, newton_iters, launches;
    long long net_armed_solves;   // solves enqueued with the network's conditional correction
};

namespace qd {
// mg.cu
// jrow: the depth metric per staggered row of mu_equi (2nz-1 values), or null
int mg_alloc(qd_solver *s, const double *mu_equi_host, const double *jrow_host);
void mg_free(qd_solver *s);
int mg_solve(qd_solver *s, int *cycles, double *rnorm, double *r0norm);
int mg_smooth(qd_solver *s, int level, int nsweeps);
int mg_vcycle(qd_solver *s);
int mg_residual_norm(qd_solver *s, double *rnorm);
int build_coarse_inverse(qd_solver *s);
// mg_fused.cu
int vcycle64_norm(qd_solver *s, int *nblocks);
int vcycle32_into64(qd_solver *s);
int smooth32_into64(qd_solver *s);
void tma_cache_free(qd_solver *s);
int tail_image_build(qd_solver *s);
int tiles_set(qd_solver *s, int box_up, int box_down);
void tiles_default_level0(const qd_solver *s, int *box_up, int *box_down);
int time_kernel(qd_solver *s, int which, int reps, double *us);
// a bounded mbarrier wait that nothing completes (gives up after `polls`)
int wait_probe(qd_solver *s, unsigned polls);
// mg.cu: level-0 norms into d_scal[slot] (to32: the mixed solver's
// double-float residual -> FP32 rhs)
int level0_norm(qd_solver *s, int to32, int slot);
int level0_norm_decide(qd_solver *s, const Decide &dc);
// u = u0 + alpha (u - u0) with the alpha that minimises the energy norm of
// the level-0 error (the guess u0's correction u - u0 scaled optimally)
int mr_step(qd_solver *s, const double *u0);
int convert_f64_f32(const double *in, float *out, int n, float *lo = nullptr);
int r0_norm(qd_solver *s, int slot);
void tail_image_free(qd_solver *s);
// mg_graph.cu
int mg_solve_async(qd_solver *s);
int solve_state_read(qd_solver *s, SolveState *out);
int solve_state_clear_flag(qd_solver *s);
void solve_graph_free(qd_solver *s);
// unet.cu: the warm start's standby decision from an RK attempt's need_max
void warm_start_standby_update(qd_solver *s, double need_max);
// fault.cu
int fault_alloc(qd_solver *s);
void fault_free(qd_solver *s);
// fit: also fit the new boundary data by the solution history's (when the
// next solve will start from a history guess), for history_apply
// commit: the accepted step's commit first (stage 1's refresh)
int launch_stage_boundary(qd_solver *s, int stage, double ratio, bool fit, bool commit = false);
// a copy of the solved level-0 u into a slot of the solution history
// (history_push_job), run by extra CTAs of the fault-stage kernel
struct CopyJob {
    const double *src = nullptr;   // null: no copy
    float2 *dst = nullptr;         // N x P field as double-float pairs (d_split)
    double *bc = nullptr;          // its boundary columns, [fault rows, far rows]
    int N = 0, K = 0, P = 0;
};
// the stage's stress, Newton and aging law (k_fault_stage); with job.src
// set the same launch also stores u into the solution history
int launch_fault(qd_solver *s, int stage, const CopyJob &job);
// the error estimate; with report set, its last block also writes the
// attempt's report (the error, the solve state, the status) straight into
// the solver's pinned host copies, in place of three copies after it
int launch_error(qd_solver *s, bool report);
int launch_stress(qd_solver *s);
int launch_newton(qd_solver *s, const double *Ts, const double *psi, double *V, int *iters);
int launch_dpsi(qd_solver *s, const double *psi, const double *V, double *dpsi);
void rk_tableau(double c[7], double b[7], double hb[7], double a[7][7]);
// medium.cu
int set_medium_gpu(int ni, int nk, const double *mu_node, double *mu_equi);
// unet.cu: the learned warm start around a stage solve
int warm_start_before_boundary(qd_solver *s);
int warm_start_after_boundary(qd_solver *s);
int warm_start_after_solve(qd_solver *s);
// true while a network in prediction mode is attached: each solve then
// corrects its guess with warm_start_predict when the guess misses the
// tolerance (a conditional node of the solve graph)
bool warm_start_predicting(qd_solver *s);
// the network's correction of the guess in u (enqueued on the solver's
// stream, capturable); *kernels: the kernels it launched that s->launches
// does not count
int warm_start_predict(qd_solver *s, int *kernels);
void warm_start_detach(qd_solver *s);
double *warm_start_bc_buffer(qd_solver *s);
// history.cu: initial guess from the solution history
int history_set(qd_solver *s, int m);
// the guess in u's interior from the fit launch_stage_boundary made
// (no-op without one)
int history_apply(qd_solver *s, double *implied_bc);
// after a stage solve: the store of the solution into the ring as a copy
// job for the next kernel that takes one (the ring's slot is claimed now);
// job->src stays null without a history
int history_push_job(qd_solver *s, CopyJob *job);
void history_reset(qd_solver *s);
void history_free(qd_solver *s);
int history_last_fit(qd_solver *s, double *out, int *nd);
bool history_will_guess(qd_solver *s);
int history_replay_guess(qd_solver *s);
// autotune.cu
int autotune(qd_solver *s, int reps, qd_tuning *out);
// io.cu
void snapshot_free(qd_solver *s);
}  // namespace qd
