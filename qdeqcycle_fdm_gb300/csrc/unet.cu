// unet.cu -- the learned warm start: a 4-level BF16 U-Net (16/32/64/128
// channels, 3x3 convolutions, FP32 accumulation) that predicts the change of
// the displacement field a stage solve will make, trained online on the
// multigrid's own solutions with hand-written tcgen05 forward, data-gradient
// and weight-gradient kernels (unet_conv.cuh) and an Adam update.
//
// Network (levels 0..3 at N, (N-1)/2+1, ... nodes; every conv 3x3 + bias):
//   e0a = relu(conv(x0)) ; e0 = relu(conv(e0a))                16 ch
//   e1a = relu(conv(pool(e0))) ; e1 = relu(conv(e1a))          32 ch
//   e2a = relu(conv(pool(e1))) ; e2 = relu(conv(e2a))          64 ch
//   e3a = relu(conv(pool(e2))) ; e3 = relu(conv(e3a))         128 ch
//   d2 = relu(conv(relu(conv(up(e3))) + e2))                   64 ch
//   d1 = relu(conv(relu(conv(up(d2))) + e1))                   32 ch
//   d0 = relu(conv(relu(conv(up(d1))) + e0))                   16 ch
//   out = conv(d0) channel 0                                   (FP32)
// pool: mean of the 2x2 fine nodes (2i..2i+1, 2j..2j+1) inside the grid;
// up: bilinear, the multigrid prolongation's weights.
//
// Input channels (x0, padded to 16): u/s_u, d_fault/s_bc broadcast along
// each row, d_far/s_bc, the column position k/(K-1), and the change the
// previous solve made to u divided by its own s_bc; d_fault and d_far are the
// stage's change of the Dirichlet data on the fault and far columns, s_bc
// the largest of their magnitudes and s_u the largest boundary value.  The
// prediction of the change of u is s_bc * out.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <utility>
#include <vector>

#include "qdeq_internal.cuh"
#include "unet_conv.cuh"
#include "../../include/qdeq_unet.h"

namespace qd {

static constexpr int UNET_NIN = 5;   // input channels in use (of the 16 staged)
static constexpr int UNET_BIAS_BLOCKS = 1024;   // blocks of the bias-gradient sums

__host__ __device__ static inline int cdv(long a, long b) { return (int)((a + b - 1) / b); }

struct UGrid {
    int H, W, Wp, P;
};

struct UTensor {
    __nv_bfloat16 *p = nullptr;
    int C = 0, lvl = 0;
};

struct ULayer {
    int cin, cout, lvl, relu;
    UTensor *in, *out;                 // forward input / output
    UTensor *gin, *gout;               // their gradients (gin null: not needed)
    float *w32, *b32, *mw, *vw, *mb, *vb, *gw, *gb;
    __nv_bfloat16 *w, *wt;             // [9][cout][cin], [9][cin][cout]
    CUtensorMap m_in, m_w, m_gout, m_wt;   // A/B operands of forward and data gradient
    CUtensorMap m_in_rows, m_gout_rows;    // A operands as pixel-row boxes of k_conv_rows
    bool rows_fwd, rows_dgrad;             // which of the two have them
};

enum UOpKind { OP_CONV, OP_POOL, OP_UP, OP_ADD };
struct UOp {
    UOpKind k;
    int layer;                 // OP_CONV
    UTensor *a, *b, *out;      // OP_POOL/UP: a -> out; OP_ADD: a + b -> out
    UTensor *ga, *gb, *gout;
};

}  // namespace qd

struct qd_unet {
    qd::UGrid g[4];
    int nk, ni;
    std::vector<qd::ULayer> L;
    std::vector<qd::UOp> ops;
    std::vector<qd::UTensor *> acts, grads;
    qd::UTensor *x0, *head_gout;
    float *out32, *target32;       // P0 floats
    float *d_prev;                 // the last solve's change of u / s_bc (P0 floats): input channel 4
    float *d_loss;                 // [0] loss sum
    float *d_scale;                // [0] s_bc, [1] s_u, [2] 1/s_bc, [3] 1/s_u
    float *d_rowf;                 // per-row input channels: fault (N), far (N)
    double *d_bc_old;              // saved boundary columns: fault (N), far (N)
    double *d_u_start;             // u a solve would start from without the network (level-0 layout)
    __nv_bfloat16 *planar;         // dY planar + 3 shifted X planar copies
    float *parts;                  // per-CTA partial sums of a weight or bias gradient
    size_t planar_elems;
    unsigned *d_status;
    cudaStream_t stream;           // the stream the net runs on (the solver's while attached)
    cudaStream_t own_stream;
    long long steps;
    double last_loss;
    float lr;
    int mode;                      // 0 off, 1 train, 2 predict
    int stride;                    // solver level-0 nodes per network pixel (1; 2 or 4: the level-1 or -2 grid)
    bool pdl;                      // launch with programmatic stream serialization (inside forward())
};

namespace qd {

// ---------------------------------------------------------------------------
// elementwise kernels (BF16 NHWC on padded grids)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool uin(int r, int c, const UGrid &g) {
    return r >= 1 && r <= g.H && c >= 1 && c <= g.W;
}

// Eight channels per thread (C is a multiple of 8): 16-byte loads and
// stores, the pixel index from one 32-bit division per thread.
struct F8 {
    float v[8];
};

__device__ __forceinline__ F8 ld8(const __nv_bfloat16 *p) {
    const uint4 u = *reinterpret_cast<const uint4 *>(p);
    const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
    F8 f;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float2 t = __bfloat1622float2(h[i]);
        f.v[2 * i] = t.x;
        f.v[2 * i + 1] = t.y;
    }
    return f;
}

__device__ __forceinline__ void st8(__nv_bfloat16 *p, const F8 &f) {
    uint4 u;
    __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&u);
#pragma unroll
    for (int i = 0; i < 4; i++) h[i] = __floats2bfloat162_rn(f.v[2 * i], f.v[2 * i + 1]);
    *reinterpret_cast<uint4 *>(p) = u;
}

__device__ __forceinline__ void axpy8(F8 &y, float a, const F8 &x) {
#pragma unroll
    for (int i = 0; i < 8; i++) y.v[i] += a * x.v[i];
}

// 2x2 mean pool, fine level f -> coarse level c
__global__ void k_pool(const __nv_bfloat16 *in, __nv_bfloat16 *out, UGrid f, UGrid c, int C) {
    pdl_trigger();
    pdl_wait();
    const int C8 = C >> 3, idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= c.P * C8) return;
    const int p = idx / C8, ch = (idx - p * C8) * 8;
    const int r = p / c.Wp, q = p - r * c.Wp;
    F8 v = {};
    if (uin(r, q, c)) {
        const int y0 = 2 * (r - 1), x0 = 2 * (q - 1);
        int n = 0;
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
                if (y0 + a < f.H && x0 + b < f.W) {
                    axpy8(v, 1.f, ld8(in + ((long)(y0 + a + 1) * f.Wp + (x0 + b + 1)) * C + ch));
                    n++;
                }
        const float w = n == 4 ? 0.25f : (n == 2 ? 0.5f : 1.f);   // exact: the mean of 1, 2 or 4 nodes
#pragma unroll
        for (int i = 0; i < 8; i++) v.v[i] *= w;
    }
    st8(out + (long)p * C + ch, v);
}

// gradient of k_pool, added into gin (fine)
__global__ void k_pool_bwd(const __nv_bfloat16 *gout, __nv_bfloat16 *gin, UGrid f, UGrid c, int C) {
    const int C8 = C >> 3, idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= f.P * C8) return;
    const int p = idx / C8, ch = (idx - p * C8) * 8;
    const int r = p / f.Wp, q = p - r * f.Wp;
    if (!uin(r, q, f)) return;
    const int y = r - 1, x = q - 1, yc = y >> 1, xc = x >> 1;
    const int ny = (2 * yc + 1 < f.H) ? 2 : 1, nx = (2 * xc + 1 < f.W) ? 2 : 1;
    F8 g = ld8(gin + (long)p * C + ch);
    axpy8(g, 1.f / (float)(ny * nx), ld8(gout + ((long)(yc + 1) * c.Wp + (xc + 1)) * C + ch));
    st8(gin + (long)p * C + ch, g);
}

// bilinear up-sampling, coarse c -> fine f: one thread per coarse node and
// eight channels writes the 2 x 2 fine block the node starts (the block is
// clipped at the last fine row and column).  The fine border pixels are not
// written: the tensor is zeroed at allocation and only this kernel writes it.
__global__ void k_up(const __nv_bfloat16 *in, __nv_bfloat16 *out, UGrid c, UGrid f, int C) {
    pdl_trigger();
    pdl_wait();
    const int C8 = C >> 3;
    const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (idx >= (long)c.H * c.W * C8) return;
    const long cell = idx / C8;
    const int ch = (int)(idx - cell * C8) * 8;
    const int yc = (int)(cell / c.W), xc = (int)(cell - (long)yc * c.W);
    const bool hy = 2 * yc + 1 < f.H, hx = 2 * xc + 1 < f.W;
    const __nv_bfloat16 *b = in + ((long)(yc + 1) * c.Wp + (xc + 1)) * C + ch;
    const long dn = (long)c.Wp * C, fdn = (long)f.Wp * C;
    const F8 a = ld8(b);
    const F8 bx = hx ? ld8(b + C) : a, by = hy ? ld8(b + dn) : a;
    __nv_bfloat16 *o = out + ((long)(2 * yc + 1) * f.Wp + (2 * xc + 1)) * C + ch;
    st8(o, a);
    F8 v;
    if (hx) {
#pragma unroll
        for (int i = 0; i < 8; i++) v.v[i] = 0.5f * a.v[i] + 0.5f * bx.v[i];
        st8(o + C, v);
    }
    if (hy) {
#pragma unroll
        for (int i = 0; i < 8; i++) v.v[i] = 0.5f * a.v[i] + 0.5f * by.v[i];
        st8(o + fdn, v);
        if (hx) {
            const F8 bxy = ld8(b + dn + C);
#pragma unroll
            for (int i = 0; i < 8; i++) {
                float t = 0.f;
                t += 0.25f * a.v[i];
                t += 0.25f * by.v[i];
                t += 0.25f * bx.v[i];
                t += 0.25f * bxy.v[i];
                v.v[i] = t;
            }
            st8(o + fdn + C, v);
        }
    }
}

// gradient of k_up (its transpose), written into gin (coarse)
__global__ void k_up_bwd(const __nv_bfloat16 *gout, __nv_bfloat16 *gin, UGrid c, UGrid f, int C) {
    const int C8 = C >> 3, idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= c.P * C8) return;
    const int p = idx / C8, ch = (idx - p * C8) * 8;
    const int r = p / c.Wp, q = p - r * c.Wp;
    F8 v = {};
    if (uin(r, q, c)) {
        const int y = 2 * (r - 1), x = 2 * (q - 1);
        for (int dy = -1; dy <= 1; dy++) {
            const int yy = y + dy;
            if (yy < 0 || yy >= f.H) continue;
            const float wy = dy ? 0.5f : 1.f;
            for (int dx = -1; dx <= 1; dx++) {
                const int xx = x + dx;
                if (xx < 0 || xx >= f.W) continue;
                axpy8(v, wy * (dx ? 0.5f : 1.f), ld8(gout + ((long)(yy + 1) * f.Wp + (xx + 1)) * C + ch));
            }
        }
    }
    st8(gin + (long)p * C + ch, v);
}

// the element kernels below take n = pixels * channels (a multiple of 8)
__global__ void k_add(const __nv_bfloat16 *a, const __nv_bfloat16 *b, __nv_bfloat16 *out, long n) {
    pdl_trigger();
    pdl_wait();
    const long i = 8L * (blockIdx.x * (long)blockDim.x + threadIdx.x);
    if (i >= n) return;
    F8 x = ld8(a + i);
    axpy8(x, 1.f, ld8(b + i));
    st8(out + i, x);
}

__global__ void k_copy2(const __nv_bfloat16 *g, __nv_bfloat16 *a, __nv_bfloat16 *b, long n) {
    const long i = 8L * (blockIdx.x * (long)blockDim.x + threadIdx.x);
    if (i >= n) return;
    const uint4 u = *reinterpret_cast<const uint4 *>(g + i);
    *reinterpret_cast<uint4 *>(a + i) = u;
    *reinterpret_cast<uint4 *>(b + i) = u;
}

// g *= (y > 0), in place
__global__ void k_relu_bwd(__nv_bfloat16 *g, const __nv_bfloat16 *y, long n) {
    const long i = 8L * (blockIdx.x * (long)blockDim.x + threadIdx.x);
    if (i >= n) return;
    F8 gv = ld8(g + i);
    const F8 yv = ld8(y + i);
#pragma unroll
    for (int k = 0; k < 8; k++)
        if (!(yv.v[k] > 0.f)) gv.v[k] = 0.f;
    st8(g + i, gv);
}

// NHWC [P][C] -> planar [C][P], shifted by dx pixels (zero outside)
__global__ void k_planar(const __nv_bfloat16 *in, __nv_bfloat16 *out, int P, int C, int dx) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)P * C) return;
    const int c = (int)(idx / P), p = (int)(idx - (long)c * P), s = p + dx;
    out[idx] = (s >= 0 && s < P) ? in[(long)s * C + c] : __float2bfloat16_rn(0.f);
}

// per-channel sum of g over a block's share of the pixels (bias gradient):
// thread (lane l, channel c) of the block sums pixels p0 + l, p0 + l + L, ...
// in order, the lanes are then added in order; part[block][c]
__global__ void __launch_bounds__(256) k_bias_grad(const __nv_bfloat16 *g, float *part, int P, int C) {
    __shared__ float acc[256];
    const int L = blockDim.x / C, c = threadIdx.x % C, l = threadIdx.x / C;
    const int per = cdv(P, gridDim.x);
    const int p0 = blockIdx.x * per, p1 = min(P, p0 + per);
    float s = 0.f;
    if (l < L)
        for (int p = p0 + l; p < p1; p += L) s += __bfloat162float(g[(long)p * C + c]);
    acc[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < C) {
        float t = 0.f;
        for (int k = 0; k < L; k++) t += acc[k * C + threadIdx.x];
        part[(size_t)blockIdx.x * C + threadIdx.x] = t;
    }
}

// Adam on one layer's FP32 master weights and biases, then the BF16 copies
__global__ void k_adam(ULayer L, float lr, float b1, float b2, float c1, float c2, float eps) {
    const int nw = 9 * L.cout * L.cin;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nw) {
        const float g = L.gw[i];
        const float m = b1 * L.mw[i] + (1.f - b1) * g, v = b2 * L.vw[i] + (1.f - b2) * g * g;
        L.mw[i] = m;
        L.vw[i] = v;
        const float w = L.w32[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
        L.w32[i] = w;
        const int t = i / (L.cout * L.cin), r = i - t * L.cout * L.cin, co = r / L.cin, ci = r - co * L.cin;
        L.w[i] = __float2bfloat16_rn(w);
        L.wt[((long)t * L.cin + ci) * L.cout + co] = __float2bfloat16_rn(w);
    } else if (i < nw + L.cout) {
        const int j = i - nw;
        const float g = L.gb[j];
        const float m = b1 * L.mb[j] + (1.f - b1) * g, v = b2 * L.vb[j] + (1.f - b2) * g * g;
        L.mb[j] = m;
        L.vb[j] = v;
        L.b32[j] = L.b32[j] - lr * (m / c1) / (sqrtf(v / c2) + eps);
    }
}

// BF16 copies of the FP32 master weights
__global__ void k_weights_bf16(ULayer L) {
    const int nw = 9 * L.cout * L.cin;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nw) return;
    const int t = i / (L.cout * L.cin), r = i - t * L.cout * L.cin, co = r / L.cin, ci = r - co * L.cin;
    L.w[i] = __float2bfloat16_rn(L.w32[i]);
    L.wt[((long)t * L.cin + ci) * L.cout + co] = __float2bfloat16_rn(L.w32[i]);
}

// mean squared error over the interior; gradient into channel 0 of gout
// (16 channels), loss sum into *loss
__global__ void k_loss(const float *out, const float *target, __nv_bfloat16 *gout, float *loss, UGrid g,
                       float inv_n) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (p < g.P) {
        const int r = p / g.Wp, q = p - r * g.Wp;
        float gr = 0.f;
        if (uin(r, q, g)) {
            const float d = out[p] - target[p];
            l = d * d * inv_n;
            gr = 2.f * d * inv_n;
        }
        gout[(long)p * 16] = __float2bfloat16_rn(gr);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// ---------------------------------------------------------------------------
// solver coupling (level-0 field u: N rows x K columns, pitch P)
// ---------------------------------------------------------------------------
__global__ void k_save_bc(const double *u, int N, int K, int P, double *bc) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    bc[j] = u[(long)j * P];
    bc[N + j] = u[(long)j * P + K - 1];
}

// One CTA over the boundary rows: s_bc = max |change of the boundary data|,
// s_u = max |boundary data|, their reciprocals, and the two per-row input
// channels (change on the fault / far column over s_bc).  Every row's
// difference is taken in FP64 and rounded to FP32 on the integer pipes
// (d2f_rne); scales and features are FP32 (the network's inputs are BF16).
// scale: [0] s_bc, [1] s_u, [2] 1/s_bc, [3] 1/s_u; rowf: fault (N), far (N)
__global__ void __launch_bounds__(1024) k_scales(const double *u, int N, int K, int P, const double *bc,
                                                 float *scale, float *rowf) {
    __shared__ float wb[32], wu[32], inv[2];
    float sb = 0.f, su = 0.f;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const double f = u[(long)j * P], r = u[(long)j * P + K - 1];
        const float df = d2f_rne(f - bc[j]), dr = d2f_rne(r - bc[N + j]);
        rowf[j] = df;
        rowf[N + j] = dr;
        sb = fmaxf(sb, fmaxf(fabsf(df), fabsf(dr)));
        su = fmaxf(su, fmaxf(fabsf(d2f_rne(f)), fabsf(d2f_rne(r))));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sb = fmaxf(sb, __shfl_xor_sync(0xffffffffu, sb, o));
        su = fmaxf(su, __shfl_xor_sync(0xffffffffu, su, o));
    }
    if ((threadIdx.x & 31) == 0) {
        wb[threadIdx.x >> 5] = sb;
        wu[threadIdx.x >> 5] = su;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            sb = fmaxf(sb, wb[w]);
            su = fmaxf(su, wu[w]);
        }
        sb = fmaxf(sb, 1e-30f);
        su = fmaxf(su, 1e-30f);
        scale[0] = sb;
        scale[1] = su;
        scale[2] = inv[0] = 1.f / sb;
        scale[3] = inv[1] = 1.f / su;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += blockDim.x) {   // each thread rescales the rows it wrote
        rowf[j] *= inv[0];
        rowf[N + j] *= inv[0];
    }
}

// input channels at network pixel (r, q): the solver's level-0 node
// (st (r-1), st (q-1)) -- every node (st = 1), every other one (st = 2, the
// network on the multigrid's level-1 grid) or every fourth (st = 4, level 2)
__global__ void k_features(const double *u, int N, int K, int P, const float *rowf, const float *scale,
                           const float *prev, __nv_bfloat16 *x0, UGrid g, int st) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= g.P) return;
    const int r = p / g.Wp, q = p - r * g.Wp;
    float f[UNET_NIN] = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (uin(r, q, g)) {
        const int j = st * (r - 1), k = st * (q - 1);
        f[0] = d2f_rne(u[(long)j * P + k]) * scale[3];
        f[1] = rowf[j];
        f[2] = rowf[N + j];
        f[3] = (float)k / (float)(K - 1);
        f[4] = prev[p];
    }
    uint4 lo, hi = make_uint4(0, 0, 0, 0);
    __nv_bfloat162 *lv = reinterpret_cast<__nv_bfloat162 *>(&lo);
    lv[0] = __floats2bfloat162_rn(f[0], f[1]);
    lv[1] = __floats2bfloat162_rn(f[2], f[3]);
    lv[2] = __floats2bfloat162_rn(f[4], 0.f);
    lv[3] = __floats2bfloat162_rn(0.f, 0.f);
    uint4 *dst = reinterpret_cast<uint4 *>(x0 + (long)p * 16);
    dst[0] = lo;
    dst[1] = hi;
}

// u0 = u on every column (the field the solve would have started from),
// then u += s_bc * out on the interior columns; with st = 2 or 4 the
// network's output on the level-1 or level-2 grid is interpolated
// bilinearly (for st = 2 these are the multigrid's prolongation weights:
// the coincident node, or the mean of the 2 or 4 neighbouring nodes)
__global__ void k_apply(double *u, double *u0, int N, int K, int P, const float *out, const float *scale, UGrid g,
                        int st) {
    const int j = blockIdx.y, k = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N || k > K - 1) return;
    const long c = (long)j * P + k;
    const double uc = u[c];
    u0[c] = uc;
    if (k == 0 || k == K - 1) return;
    float v;
    if (st == 1) {
        v = out[(long)(j + 1) * g.Wp + (k + 1)];
    } else {
        // (jc, kc): the coarse node at or before (j, k); the weights of the
        // next coarse row / column are fy / fx (zero on a coincident node,
        // whose neighbour is then not read)
        const int jc = j / st, kc = k / st;
        const float fy = (float)(j - jc * st) / (float)st, fx = (float)(k - kc * st) / (float)st;
        const float *o = out + (long)(jc + 1) * g.Wp + (kc + 1);
        const float r0 = fx > 0.f ? (1.f - fx) * o[0] + fx * o[1] : o[0];
        if (fy > 0.f) {
            const float r1 = fx > 0.f ? (1.f - fx) * o[g.Wp] + fx * o[g.Wp + 1] : o[g.Wp];
            v = (1.f - fy) * r0 + fy * r1;
        } else {
            v = r0;
        }
    }
    u[c] = uc + (double)scale[0] * (double)v;
}

// training target: (u_solved - u_start) / s_bc on the interior (the
// difference in FP64, then FP32); zero when `ss` says the network did not
// run on this solve (u_start is then not this solve's starting field: the
// gate keeps it only when the network corrects the guess)
__global__ void k_target(const double *u, const double *u0, int N, int K, int P, const float *scale,
                         float *target, UGrid g, int st, const SolveState *ss) {
    pdl_trigger();
    pdl_wait();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= g.P) return;
    const int r = p / g.Wp, q = p - r * g.Wp;
    float t = 0.f;
    if (uin(r, q, g) && (!ss || ss->net)) {
        const long c = (long)st * (r - 1) * P + (long)st * (q - 1);
        t = d2f_rne(u[c] - u0[c]) * scale[2];
    }
    target[p] = t;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int swz(int row_bytes) {
    return row_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                            : (row_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
}

// A operand of a convolution: NHWC activation [P][C], box KB x 128
static int map_act(CUtensorMap *m, const UTensor &t, const UGrid &g) {
    const int KB = t.C < 64 ? t.C : 64;
    return encode_tiled_2d(m, t.p, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, t.C, g.P, (long)t.C * 2, KB, 128,
                           swz(KB * 2));
}

// A operand of k_conv_rows: the tensor as (channel, column, row) with boxes
// of all C channels x 130 columns x (mt + 2) rows, mt the convolution's tile
// height, swizzled to the pixel row (32 or 64 bytes)
static int map_act_rows(CUtensorMap *m, const UTensor &t, const UGrid &g, int mt) {
    return encode_tiled_3d(m, t.p, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, t.C, g.Wp, g.H + 2, (long)t.C * 2,
                           (long)g.Wp * t.C * 2, t.C, ROWS_BOXW, mt + 2, swz(t.C * 2));
}

// tile height of k_conv_rows for cin -> cout channels (0: not a row-box case)
static int rows_mt(int cin, int cout) {
#define QD_MT_CASE(ci, co) \
    if (cin == ci && cout == co) return conv_rows_mt<ci, co>();
    QD_MT_CASE(16, 16) QD_MT_CASE(16, 32) QD_MT_CASE(16, 64)
    QD_MT_CASE(32, 16) QD_MT_CASE(32, 32) QD_MT_CASE(32, 64)
    QD_MT_CASE(64, 32) QD_MT_CASE(64, 64)
#undef QD_MT_CASE
    return 0;
}

// B operand: weights [9*rows][K], box KB x rows
static int map_w(CUtensorMap *m, const __nv_bfloat16 *w, int rows, int K) {
    const int KB = K < 64 ? K : 64;
    return encode_tiled_2d(m, w, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, K, 9L * rows, (long)K * 2, KB, rows,
                           swz(KB * 2));
}

static int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
            n = 1;
    }
    return n;
}

template <int KB, int COUT, int MT_>
static int conv_launch_mt(qd_unet *u, const CUtensorMap &ta, const CUtensorMap &tb, const ConvArgs &a) {
    constexpr int MT = MT_ ? MT_ : conv_mt<KB, COUT>();
    constexpr int STAGE = ((MT * 128 * KB * 2 + COUT * KB * 2) + 1023) / 1024 * 1024;
    const size_t smem = (size_t)CONV_STAGES * STAGE + 1024;
    static bool raised = false;
    if (!raised) {
        QD_CUDA(cudaFuncSetAttribute(k_conv_fwd<KB, COUT, MT_>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
        raised = true;
    }
    QD_CUDA(launch_pdl(u->pdl, k_conv_fwd<KB, COUT, MT_>, dim3(cdv(a.P, 128 * MT)), dim3(CONV_THREADS), smem,
                     u->stream, ta, tb, a));
    QD_CUDA(cudaPeekAtLastError());
    return QD_OK;
}

// one sub-tile per CTA where MT-tile CTAs would leave SMs idle
template <int KB, int COUT>
static int conv_launch(qd_unet *u, const CUtensorMap &ta, const CUtensorMap &tb, const ConvArgs &a) {
    constexpr int MT = conv_mt<KB, COUT>();
    if (MT > 1 && cdv(a.P, 128 * MT) < sm_count()) return conv_launch_mt<KB, COUT, 1>(u, ta, tb, a);
    return conv_launch_mt<KB, COUT, 0>(u, ta, tb, a);
}


// CTAs of a kernel that fit on one SM at once, from its attributes: shared
// memory (static + dynamic + the 1 KB the driver reserves per CTA),
// registers (allocated per warp in units of 256), threads, and tensor-memory
// columns (512 per SM)
static int ctas_per_sm(const void *fn, int threads, size_t dyn_smem, int tmem_cols) {
    cudaFuncAttributes fa{};
    int dev = 0, smem_sm = 0, regs_sm = 0, thr_sm = 0;
    if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev) != cudaSuccess)
        return 1;
    const long smem_cta = (long)fa.sharedSizeBytes + (long)dyn_smem + 1024;
    const int warps = (threads + 31) / 32;
    const long regs_cta = (long)warps * (((long)fa.numRegs * 32 + 255) / 256 * 256);
    long n = smem_sm / smem_cta;
    n = std::min(n, regs_sm / std::max(1L, regs_cta));
    n = std::min(n, (long)(thr_sm / threads));
    n = std::min(n, (long)(512 / tmem_cols));
    return (int)std::max(1L, n);
}

// persistent: as many CTAs as fit on the GPU at once, at most one per tile
template <int CIN, int COUT>
static int conv_rows_launch(qd_unet *u, const CUtensorMap &ta, const CUtensorMap &tb, const ConvArgs &a) {
    using R = RowsCfg<CIN, COUT>;
    static int per_sm = 0;
    if (!per_sm) {
        QD_CUDA(cudaFuncSetAttribute(k_conv_rows<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)R::SMEM));
        QD_CUDA(cudaFuncSetAttribute(k_conv_rows<CIN, COUT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared));
        per_sm = ctas_per_sm((const void *)k_conv_rows<CIN, COUT>, ROWS_THREADS, R::SMEM, (int)R::TCOLS);
    }
    const int tiles = cdv(a.H + 2, R::MT) * cdv(a.Wp, 128);
    const int grid = std::min(tiles, per_sm * sm_count());
    QD_CUDA(launch_pdl(u->pdl, k_conv_rows<CIN, COUT>, dim3(grid), dim3(ROWS_THREADS), R::SMEM, u->stream, ta, tb, a));
    QD_CUDA(cudaPeekAtLastError());
    return QD_OK;
}

// ta_rows: the row-box map of the A operand (16, 32 or 64 channels), or null
static int conv_dispatch(qd_unet *u, const CUtensorMap &ta, const CUtensorMap *ta_rows, const CUtensorMap &tb,
                         const ConvArgs &a) {
    if (ta_rows) {
#define QD_ROWS_CASE(ci, co) \
    if (a.Cin == ci && a.Cout == co) return conv_rows_launch<ci, co>(u, *ta_rows, tb, a);
        QD_ROWS_CASE(16, 16) QD_ROWS_CASE(16, 32) QD_ROWS_CASE(16, 64)
        QD_ROWS_CASE(32, 16) QD_ROWS_CASE(32, 32) QD_ROWS_CASE(32, 64)
        QD_ROWS_CASE(64, 32) QD_ROWS_CASE(64, 64)
#undef QD_ROWS_CASE
    }
    const int KB = a.Cin < 64 ? a.Cin : 64;
#define QD_CONV_CASE(kb, co) \
    if (KB == kb && a.Cout == co) return conv_launch<kb, co>(u, ta, tb, a);
    QD_CONV_CASE(16, 16) QD_CONV_CASE(16, 32) QD_CONV_CASE(16, 64) QD_CONV_CASE(16, 128)
    QD_CONV_CASE(32, 16) QD_CONV_CASE(32, 32) QD_CONV_CASE(32, 64) QD_CONV_CASE(32, 128)
    QD_CONV_CASE(64, 16) QD_CONV_CASE(64, 32) QD_CONV_CASE(64, 64) QD_CONV_CASE(64, 128)
#undef QD_CONV_CASE
    set_error("no convolution kernel for %d -> %d channels", a.Cin, a.Cout);
    return QD_ERR_ARG;
}

template <int CIN>
static int wgrad_launch(qd_unet *u, const WgradMaps &m, const WgradArgs &a, int nchunks) {
    constexpr int STAGE = ((128 * 128 + CIN * 128) + 1023) / 1024 * 1024;
    const size_t smem = (size_t)CONV_STAGES * STAGE + 1024;
    static bool raised = false;
    if (!raised) {
        QD_CUDA(cudaFuncSetAttribute(k_conv_wgrad<CIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
        raised = true;
    }
    k_conv_wgrad<CIN><<<dim3(nchunks, 9), CONV_THREADS, smem, u->stream>>>(m, a);
    QD_CUDA(cudaPeekAtLastError());
    return QD_OK;
}

static ConvArgs conv_args(const qd_unet *u, const UGrid &g, int cin, int cout) {
    ConvArgs a;
    memset(&a, 0, sizeof(a));
    a.Cin = cin; a.Cout = cout; a.KB = cin < 64 ? cin : 64;
    a.Wp = g.Wp; a.H = g.H; a.W = g.W; a.P = g.P;
    a.status = u->d_status;
    return a;
}

#define EW_GRID(n) cdv((long)(n), 256), 256, 0, u->stream
#define EW8_GRID(n) cdv((long)(n) / 8, 256), 256, 0, u->stream   // eight channels per thread

// forward through every layer; the head writes out32.  Its kernels are
// launched with programmatic stream serialization: each one's set-up
// overlaps the previous one's tail, and it waits for the previous one's
// results (pdl_wait) before it touches them.  The first waits on whatever
// preceded the forward pass; the next kernel after it, launched normally,
// waits for its completion.
static int forward_ops(qd_unet *u);
static int forward(qd_unet *u) {
    u->pdl = true;
    const int rc = forward_ops(u);
    u->pdl = false;
    return rc;
}

static int forward_ops(qd_unet *u) {
    for (const UOp &op : u->ops) {
        if (op.k == OP_CONV) {
            ULayer &Ly = u->L[op.layer];
            const UGrid &g = u->g[Ly.lvl];
            ConvArgs a = conv_args(u, g, Ly.cin, Ly.cout);
            a.relu = Ly.relu;
            a.bias = Ly.b32;
            if (Ly.out) a.out = Ly.out->p; else a.out_f32 = u->out32;
            QD_TRY(conv_dispatch(u, Ly.m_in, Ly.rows_fwd ? &Ly.m_in_rows : nullptr, Ly.m_w, a));
        } else if (op.k == OP_POOL) {
            const long n = (long)u->g[op.out->lvl].P * op.out->C;
            QD_CUDA(launch_pdl(true, k_pool, dim3(cdv(n / 8, 256)), dim3(256), 0, u->stream, op.a->p, op.out->p,
                             u->g[op.a->lvl], u->g[op.out->lvl], op.a->C));
        } else if (op.k == OP_UP) {
            const UGrid &gc = u->g[op.a->lvl];
            const long n = (long)gc.H * gc.W * (op.a->C / 8);
            QD_CUDA(launch_pdl(true, k_up, dim3(cdv(n, 256)), dim3(256), 0, u->stream, op.a->p, op.out->p, gc,
                             u->g[op.out->lvl], op.a->C));
        } else {
            const long n = (long)u->g[op.out->lvl].P * op.out->C;
            QD_CUDA(launch_pdl(true, k_add, dim3(cdv(n / 8, 256)), dim3(256), 0, u->stream,
                             (const __nv_bfloat16 *)op.a->p, (const __nv_bfloat16 *)op.b->p, op.out->p, n));
        }
        QD_CUDA(cudaPeekAtLastError());
    }
    return QD_OK;
}

template <int CIN>
static int wgrad_layer(qd_unet *u, ULayer &Ly) {
    const UGrid &g = u->g[Ly.lvl];
    __nv_bfloat16 *dyp = u->planar, *xp = u->planar + (size_t)128 * g.P;
    WgradMaps m;
    QD_TRY(encode_tiled_2d(&m.dy, dyp, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, g.P, Ly.cout, (long)g.P * 2, 64,
                           128, CU_TENSOR_MAP_SWIZZLE_128B));
    k_planar<<<EW_GRID((long)g.P * Ly.cout)>>>(Ly.gout->p, dyp, g.P, Ly.cout, 0);
    for (int d = 0; d < 3; d++) {
        __nv_bfloat16 *x = xp + (size_t)d * CIN * g.P;
        k_planar<<<EW_GRID((long)g.P * CIN)>>>(Ly.in->p, x, g.P, CIN, d - 1);
        QD_TRY(encode_tiled_2d(&m.x[d], x, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, g.P, CIN, (long)g.P * 2, 64,
                               CIN, CU_TENSOR_MAP_SWIZZLE_128B));
    }
    QD_CUDA(cudaPeekAtLastError());
    WgradArgs a;
    a.Cin = CIN; a.Cout = Ly.cout; a.Wp = g.Wp; a.P = g.P;
    a.chunk = 64 * 32;
    a.part = u->parts;
    a.status = u->d_status;
    const int nchunks = cdv(g.P, a.chunk);
    QD_TRY(wgrad_launch<CIN>(u, m, a, nchunks));
    const int n = 9 * Ly.cout * CIN;
    k_sum_parts<<<cdv(n, 256), 256, 0, u->stream>>>(u->parts, nchunks, n, Ly.gw);
    QD_CUDA(cudaPeekAtLastError());
    return QD_OK;
}

// gradient of the loss already in head_gout; every layer's gw/gb
static int backward(qd_unet *u) {
    for (auto *t : u->grads)
        if (t != u->head_gout)
            QD_CUDA(cudaMemsetAsync(t->p, 0, sizeof(__nv_bfloat16) * (size_t)u->g[t->lvl].P * t->C, u->stream));
    for (auto &Ly : u->L) {
        QD_CUDA(cudaMemsetAsync(Ly.gw, 0, sizeof(float) * 9 * Ly.cout * Ly.cin, u->stream));
        QD_CUDA(cudaMemsetAsync(Ly.gb, 0, sizeof(float) * Ly.cout, u->stream));
    }
    for (int i = (int)u->ops.size() - 1; i >= 0; i--) {
        const UOp &op = u->ops[i];
        if (op.k == OP_CONV) {
            ULayer &Ly = u->L[op.layer];
            const UGrid &g = u->g[Ly.lvl];
            const long n = (long)g.P * Ly.cout;
            if (Ly.relu) k_relu_bwd<<<EW8_GRID(n)>>>(Ly.gout->p, Ly.out->p, n);
            const int nb = std::min(cdv(g.P, 256), UNET_BIAS_BLOCKS);
            k_bias_grad<<<nb, 256, 0, u->stream>>>(Ly.gout->p, u->parts, g.P, Ly.cout);
            k_sum_parts<<<1, 128, 0, u->stream>>>(u->parts, nb, Ly.cout, Ly.gb);
            QD_CUDA(cudaPeekAtLastError());
            switch (Ly.cin) {
                case 16: QD_TRY(wgrad_layer<16>(u, Ly)); break;
                case 32: QD_TRY(wgrad_layer<32>(u, Ly)); break;
                case 64: QD_TRY(wgrad_layer<64>(u, Ly)); break;
                case 128: QD_TRY(wgrad_layer<128>(u, Ly)); break;
                default: set_error("no weight-gradient kernel for %d channels", Ly.cin); return QD_ERR_ARG;
            }
            if (Ly.gin) {
                ConvArgs a = conv_args(u, g, Ly.cout, Ly.cin);
                a.out = Ly.gin->p;
                a.tap_reverse = 1;
                QD_TRY(conv_dispatch(u, Ly.m_gout, Ly.rows_dgrad ? &Ly.m_gout_rows : nullptr, Ly.m_wt, a));
            }
        } else if (op.k == OP_POOL) {
            const long n = (long)u->g[op.a->lvl].P * op.a->C;
            k_pool_bwd<<<EW8_GRID(n)>>>(op.gout->p, op.ga->p, u->g[op.a->lvl], u->g[op.out->lvl], op.a->C);
        } else if (op.k == OP_UP) {
            const long n = (long)u->g[op.a->lvl].P * op.a->C;
            k_up_bwd<<<EW8_GRID(n)>>>(op.gout->p, op.ga->p, u->g[op.a->lvl], u->g[op.out->lvl], op.a->C);
        } else {
            const long n = (long)u->g[op.out->lvl].P * op.out->C;
            k_copy2<<<EW8_GRID(n)>>>(op.gout->p, op.ga->p, op.gb->p, n);
        }
        QD_CUDA(cudaPeekAtLastError());
    }
    return QD_OK;
}

static int adam(qd_unet *u) {
    u->steps++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)u->steps), c2 = 1.f - powf(b2, (float)u->steps);
    for (auto &Ly : u->L) {
        const int n = 9 * Ly.cout * Ly.cin + Ly.cout;
        k_adam<<<cdv(n, 256), 256, 0, u->stream>>>(Ly, u->lr, b1, b2, c1, c2, 1e-8f);
    }
    QD_CUDA(cudaPeekAtLastError());
    return QD_OK;
}

// loss and gradients for the target in target32 (forward included)
static int loss_and_grad(qd_unet *u) {
    QD_TRY(forward(u));
    const UGrid &g = u->g[0];
    QD_CUDA(cudaMemsetAsync(u->d_loss, 0, sizeof(float), u->stream));
    QD_CUDA(cudaMemsetAsync(u->head_gout->p, 0, sizeof(__nv_bfloat16) * (size_t)g.P * 16, u->stream));
    k_loss<<<cdv(g.P, 256), 256, 0, u->stream>>>(u->out32, u->target32, u->head_gout->p, u->d_loss, g,
                                                 1.f / ((float)g.H * (float)g.W));
    QD_CUDA(cudaPeekAtLastError());
    return backward(u);
}

static int check_unet_status(qd_unet *u) {
    unsigned st = 0;
    QD_CUDA(cudaMemcpyAsync(&st, u->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, u->stream));
    QD_CUDA(cudaStreamSynchronize(u->stream));
    if (st & ST_UNET_TIMEOUT) {
        set_error("a U-Net tensor-core kernel's pipeline wait gave up (status %u)", st);
        return QD_ERR_CUDA;
    }
    return QD_OK;
}

// deterministic normal deviates (splitmix64 + Box-Muller)
static double rnd_normal(unsigned long long *s) {
    auto next = [s]() {
        unsigned long long z = (*s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    const double u1 = ((next() >> 11) + 1.0) * (1.0 / 9007199254740993.0);
    const double u2 = (next() >> 11) * (1.0 / 9007199254740992.0);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

template <typename T>
static T *dalloc_z(size_t n, int *rc) {
    T *p = nullptr;
    if (*rc == QD_OK && (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess || cudaMemset(p, 0, n * sizeof(T)) != cudaSuccess)) {
        *rc = QD_ERR_CUDA;
        p = nullptr;
    }
    return p;
}

static void unet_free(qd_unet *u) {
    for (auto *t : u->acts) { cudaFree(t->p); delete t; }
    for (auto *t : u->grads) { cudaFree(t->p); delete t; }
    for (auto &Ly : u->L) {
        cudaFree(Ly.w32); cudaFree(Ly.b32); cudaFree(Ly.mw); cudaFree(Ly.vw); cudaFree(Ly.mb);
        cudaFree(Ly.vb); cudaFree(Ly.gw); cudaFree(Ly.gb); cudaFree(Ly.w); cudaFree(Ly.wt);
    }
    cudaFree(u->out32); cudaFree(u->target32); cudaFree(u->d_prev); cudaFree(u->d_loss); cudaFree(u->d_scale); cudaFree(u->d_rowf); cudaFree(u->parts);
    cudaFree(u->d_bc_old); cudaFree(u->d_u_start); cudaFree(u->planar); cudaFree(u->d_status);
    if (u->own_stream) cudaStreamDestroy(u->own_stream);
    delete u;
}

static int unet_build(qd_unet *u, unsigned long long seed) {
    int rc = QD_OK;
    for (int l = 0; l < 4; l++) {
        UGrid &g = u->g[l];
        g.H = l ? (u->g[l - 1].H - 1) / 2 + 1 : u->nk;
        g.W = l ? (u->g[l - 1].W - 1) / 2 + 1 : u->ni;
        g.Wp = (g.W + 2 + 7) / 8 * 8;
        g.P = (g.H + 2) * g.Wp;
    }
    auto act = [&](int C, int lvl) {
        UTensor *t = new UTensor();
        t->C = C; t->lvl = lvl;
        t->p = dalloc_z<__nv_bfloat16>((size_t)u->g[lvl].P * C, &rc);
        u->acts.push_back(t);
        return t;
    };
    auto grad = [&](UTensor *a) {
        UTensor *t = new UTensor();
        t->C = a->C; t->lvl = a->lvl;
        t->p = dalloc_z<__nv_bfloat16>((size_t)u->g[a->lvl].P * a->C, &rc);
        u->grads.push_back(t);
        return t;
    };
    auto conv = [&](UTensor *in, UTensor *gin, int cout, int relu, bool head) {
        ULayer Ly;
        memset(&Ly, 0, sizeof(Ly));
        Ly.cin = in->C; Ly.cout = cout; Ly.lvl = in->lvl; Ly.relu = relu;
        Ly.in = in; Ly.gin = gin;
        Ly.out = head ? nullptr : act(cout, in->lvl);
        Ly.gout = head ? u->head_gout : grad(Ly.out);
        const size_t nw = (size_t)9 * cout * in->C;
        Ly.w32 = dalloc_z<float>(nw, &rc); Ly.mw = dalloc_z<float>(nw, &rc);
        Ly.vw = dalloc_z<float>(nw, &rc); Ly.gw = dalloc_z<float>(nw, &rc);
        Ly.b32 = dalloc_z<float>(cout, &rc); Ly.mb = dalloc_z<float>(cout, &rc);
        Ly.vb = dalloc_z<float>(cout, &rc); Ly.gb = dalloc_z<float>(cout, &rc);
        Ly.w = dalloc_z<__nv_bfloat16>(nw, &rc); Ly.wt = dalloc_z<__nv_bfloat16>(nw, &rc);
        u->L.push_back(Ly);
        UOp op;
        memset(&op, 0, sizeof(op));
        op.k = OP_CONV; op.layer = (int)u->L.size() - 1;
        u->ops.push_back(op);
        return Ly.out;
    };
    auto pool = [&](UTensor *a, UTensor *ga) {
        UTensor *o = act(a->C, a->lvl + 1);
        UOp op;
        memset(&op, 0, sizeof(op));
        op.k = OP_POOL; op.a = a; op.out = o; op.ga = ga; op.gout = grad(o);
        u->ops.push_back(op);
        return op;
    };
    auto up = [&](UTensor *a, UTensor *ga) {
        UTensor *o = act(a->C, a->lvl - 1);
        UOp op;
        memset(&op, 0, sizeof(op));
        op.k = OP_UP; op.a = a; op.out = o; op.ga = ga; op.gout = grad(o);
        u->ops.push_back(op);
        return op;
    };
    auto add = [&](UTensor *a, UTensor *ga, UTensor *b, UTensor *gb) {
        UTensor *o = act(a->C, a->lvl);
        UOp op;
        memset(&op, 0, sizeof(op));
        op.k = OP_ADD; op.a = a; op.b = b; op.out = o; op.ga = ga; op.gb = gb; op.gout = grad(o);
        u->ops.push_back(op);
        return op;
    };
    // the gradient buffer of each layer's output is created with the layer;
    // consumers reference it through the producing layer
    auto gout_of = [&](UTensor *t) -> UTensor * {
        for (auto &Ly : u->L)
            if (Ly.out == t) return Ly.gout;
        for (auto &op : u->ops)
            if (op.out == t) return op.gout;
        return nullptr;
    };
    u->x0 = act(16, 0);
    u->head_gout = new UTensor();
    u->head_gout->C = 16; u->head_gout->lvl = 0;
    u->head_gout->p = dalloc_z<__nv_bfloat16>((size_t)u->g[0].P * 16, &rc);
    u->grads.push_back(u->head_gout);
    if (rc != QD_OK) return rc;

    UTensor *e0a = conv(u->x0, nullptr, 16, 1, false);
    UTensor *e0 = conv(e0a, gout_of(e0a), 16, 1, false);
    UOp p1 = pool(e0, gout_of(e0));
    UTensor *e1a = conv(p1.out, p1.gout, 32, 1, false);
    UTensor *e1 = conv(e1a, gout_of(e1a), 32, 1, false);
    UOp p2 = pool(e1, gout_of(e1));
    UTensor *e2a = conv(p2.out, p2.gout, 64, 1, false);
    UTensor *e2 = conv(e2a, gout_of(e2a), 64, 1, false);
    UOp p3 = pool(e2, gout_of(e2));
    UTensor *e3a = conv(p3.out, p3.gout, 128, 1, false);
    UTensor *e3 = conv(e3a, gout_of(e3a), 128, 1, false);
    UTensor *enc[3] = {e0, e1, e2};
    UTensor *cur = e3;
    for (int l = 2; l >= 0; l--) {
        const int C = enc[l]->C;
        UOp uo = up(cur, gout_of(cur));
        UTensor *da = conv(uo.out, uo.gout, C, 1, false);
        UOp ad = add(da, gout_of(da), enc[l], gout_of(enc[l]));
        cur = conv(ad.out, ad.gout, C, 1, false);
    }
    conv(cur, gout_of(cur), 16, 0, true);   // head: channel 0 is the prediction
    if (rc != QD_OK) return rc;

    // weights: He-normal, the head and the padded input channels start at zero
    unsigned long long st = seed;
    for (size_t li = 0; li < u->L.size(); li++) {
        ULayer &Ly = u->L[li];
        const bool head = li + 1 == u->L.size();
        const int cin_real = li == 0 ? UNET_NIN : Ly.cin;
        const double sd = sqrt(2.0 / (9.0 * cin_real));
        std::vector<float> w((size_t)9 * Ly.cout * Ly.cin, 0.f);
        for (int t = 0; t < 9; t++)
            for (int co = 0; co < Ly.cout; co++)
                for (int ci = 0; ci < Ly.cin; ci++) {
                    double v = rnd_normal(&st) * sd;
                    if (ci >= cin_real || head) v = 0.0;   // a fresh net predicts no change
                    w[((size_t)t * Ly.cout + co) * Ly.cin + ci] = (float)v;
                }
        QD_CUDA(cudaMemcpy(Ly.w32, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice));
        k_weights_bf16<<<cdv((long)w.size(), 256), 256, 0, u->stream>>>(Ly);
        QD_CUDA(cudaPeekAtLastError());
        QD_TRY(map_act(&Ly.m_in, *Ly.in, u->g[Ly.lvl]));
        QD_TRY(map_w(&Ly.m_w, Ly.w, Ly.cout, Ly.cin));
        QD_TRY(map_act(&Ly.m_gout, *Ly.gout, u->g[Ly.lvl]));
        Ly.rows_fwd = rows_mt(Ly.cin, Ly.cout) > 0;
        Ly.rows_dgrad = rows_mt(Ly.cout, Ly.cin) > 0;
        if (Ly.rows_fwd) QD_TRY(map_act_rows(&Ly.m_in_rows, *Ly.in, u->g[Ly.lvl], rows_mt(Ly.cin, Ly.cout)));
        if (Ly.rows_dgrad)
            QD_TRY(map_act_rows(&Ly.m_gout_rows, *Ly.gout, u->g[Ly.lvl], rows_mt(Ly.cout, Ly.cin)));
        QD_TRY(map_w(&Ly.m_wt, Ly.wt, Ly.cin, Ly.cout));
    }
    // planar scratch: dY (<= 128 rows at the layer's level) + 3 shifted X copies
    size_t need = 0;
    for (auto &Ly : u->L) need = std::max(need, (size_t)u->g[Ly.lvl].P * (128 + 3 * (size_t)Ly.cin));
    u->planar = dalloc_z<__nv_bfloat16>(need, &rc);
    u->planar_elems = need;
    // partial sums of the weight and bias gradients
    size_t nparts = 0;
    for (auto &Ly : u->L)
        nparts = std::max({nparts, (size_t)cdv(u->g[Ly.lvl].P, 64 * 32) * 9 * Ly.cout * Ly.cin,
                           (size_t)UNET_BIAS_BLOCKS * Ly.cout});
    u->parts = dalloc_z<float>(nparts, &rc);
    u->out32 = dalloc_z<float>(u->g[0].P, &rc);
    u->target32 = dalloc_z<float>(u->g[0].P, &rc);
    u->d_prev = dalloc_z<float>(u->g[0].P, &rc);
    u->d_loss = dalloc_z<float>(1, &rc);
    u->d_scale = dalloc_z<float>(4, &rc);
    // per level-0 row of the finest solver the network attaches to (four
    // times as fine: the network on its level-2 grid)
    u->d_rowf = dalloc_z<float>(2 * (4 * (size_t)u->nk - 3), &rc);
    u->d_status = dalloc_z<unsigned>(1, &rc);
    u->d_bc_old = dalloc_z<double>(2 * (4 * (size_t)u->nk - 3), &rc);
    if (rc != QD_OK) set_error("U-Net allocation failed");
    QD_CUDA(cudaStreamSynchronize(u->stream));
    return rc;
}

// host planar [C][nk][ni] float input -> x0, host [nk][ni] <-> FP32 padded
__global__ void k_x0_from_host(const float *x, int C, __nv_bfloat16 *x0, UGrid g) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= g.P) return;
    const int r = p / g.Wp, q = p - r * g.Wp;
    for (int c = 0; c < 16; c++) {
        float v = 0.f;
        if (c < C && uin(r, q, g)) v = x[((long)c * g.H + (r - 1)) * g.W + (q - 1)];
        x0[(long)p * 16 + c] = __float2bfloat16_rn(v);
    }
}

__global__ void k_pad_f32(const float *in, float *out, UGrid g) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= g.P) return;
    const int r = p / g.Wp, q = p - r * g.Wp;
    out[p] = uin(r, q, g) ? in[(long)(r - 1) * g.W + (q - 1)] : 0.f;
}

__global__ void k_unpad_f32(const float *in, float *out, UGrid g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.H * g.W) return;
    const int r = i / g.W, q = i - r * g.W;
    out[i] = in[(long)(r + 1) * g.Wp + (q + 1)];
}

static int upload_input(qd_unet *u, const float *x_host, const float *target_host) {
    const UGrid &g = u->g[0];
    const size_t n = (size_t)g.H * g.W;
    float *tmp = nullptr;
    QD_CUDA(cudaMalloc(&tmp, sizeof(float) * n * (UNET_NIN + 1)));
    int rc = QD_OK;
    if (cudaMemcpy(tmp, x_host, sizeof(float) * n * UNET_NIN, cudaMemcpyHostToDevice) != cudaSuccess ||
        (target_host &&
         cudaMemcpy(tmp + UNET_NIN * n, target_host, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess))
        rc = QD_ERR_CUDA;
    if (rc == QD_OK) {
        k_x0_from_host<<<cdv(g.P, 256), 256, 0, u->stream>>>(tmp, UNET_NIN, u->x0->p, g);
        if (target_host) k_pad_f32<<<cdv(g.P, 256), 256, 0, u->stream>>>(tmp + UNET_NIN * n, u->target32, g);
        if (cudaStreamSynchronize(u->stream) != cudaSuccess) rc = QD_ERR_CUDA;
    }
    cudaFree(tmp);
    if (rc != QD_OK) set_error("U-Net input upload failed");
    return rc;
}

}  // namespace qd

using namespace qd;

// ---------------------------------------------------------------------------
// solver coupling, called from the RK driver around each stage solve
// ---------------------------------------------------------------------------
namespace qd {

int warm_start_before_boundary(qd_solver *s) {
    qd_unet *u = static_cast<qd_unet *>(s->unet);
    if (!u || !u->mode) return QD_OK;
    if (history_will_guess(s)) return QD_OK;   // the fit writes the boundary data its guess implies
    const LevelDims &d = s->dims[0];
    k_save_bc<<<cdv(d.N, 256), 256, 0, s->stream>>>(s->L64[0].u, d.N, d.K, d.P, u->d_bc_old);
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

// the input channels of the guess now in u (k_scales, k_features)
static int features(qd_solver *s, qd_unet *u) {
    const LevelDims &d = s->dims[0];
    const UGrid &g = u->g[0];
    k_scales<<<1, 1024, 0, s->stream>>>(s->L64[0].u, d.N, d.K, d.P, u->d_bc_old, u->d_scale, u->d_rowf);
    QD_LAUNCH_CHECK(s);
    k_features<<<cdv(g.P, 256), 256, 0, s->stream>>>(s->L64[0].u, d.N, d.K, d.P, u->d_rowf, u->d_scale,
                                                     u->d_prev, u->x0->p, g, u->stride);
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

// after the new boundary data are in u, in training mode: the features, and
// the starting field for the training target (the change the solve then
// makes is the target and the next input).  In prediction mode the solve
// itself calls warm_start_predict, and only when its guess misses the
// tolerance.
int warm_start_after_boundary(qd_solver *s) {
    qd_unet *u = static_cast<qd_unet *>(s->unet);
    if (!u || u->mode != 1) return QD_OK;
    const LevelDims &d = s->dims[0];
    QD_TRY(features(s, u));
    QD_CUDA(cudaMemcpyAsync(u->d_u_start, s->L64[0].u, sizeof(double) * (size_t)d.N * d.P,
                            cudaMemcpyDeviceToDevice, s->stream));
    return QD_OK;
}

bool warm_start_predicting(qd_solver *s) {
    const qd_unet *u = static_cast<const qd_unet *>(s->unet);
    return u && u->mode == 2 && !s->net_paused && !s->net_standby;
}

// The host's side of the measured gate, once per RK attempt: when no solve
// of the attempt just finished had a first guess that needed more than
// 1 + cost V-cycles, the next attempt's solves run the graph without the
// network's conditional correction (the device gate would have left the
// network out of all of them anyway, and the conditional node itself costs
// time); as soon as one does, the network's graph comes back.  Only with the
// measured rule and in prediction mode.
void warm_start_standby_update(qd_solver *s, double need_max) {
    const qd_unet *u = static_cast<const qd_unet *>(s->unet);
    s->net_standby = u && u->mode == 2 && s->net_ratio <= 0.0 && !(need_max > 1.0 + s->net_cost);
}

// features, the forward pass and u0 = u, u += prediction (k_apply); all on
// the solver's stream, so the solve graph captures them into its IF node
int warm_start_predict(qd_solver *s, int *kernels) {
    qd_unet *u = static_cast<qd_unet *>(s->unet);
    *kernels = 0;
    if (!u || u->mode != 2) return QD_OK;
    if (u->stream != s->stream) {
        set_error("warm start: the network is attached to another solver");
        return QD_ERR_ARG;
    }
    const LevelDims &d = s->dims[0];
    QD_TRY(features(s, u));
    QD_TRY(forward(u));
    k_apply<<<dim3(cdv(d.K, 256), d.N), 256, 0, s->stream>>>(s->L64[0].u, u->d_u_start, d.N, d.K, d.P, u->out32,
                                                             u->d_scale, u->g[0], u->stride);
    QD_LAUNCH_CHECK(s);
    QD_TRY(mr_step(s, u->d_u_start));   // the prediction's energy-optimal scale: never a larger error
    *kernels = (int)u->ops.size();   // the forward pass's, one per op (not in s->launches)
    return QD_OK;
}

// the solved change (the next solve's input channel 4); in mode 1 also one
// Adam step on (features, solved change)
int warm_start_after_solve(qd_solver *s) {
    qd_unet *u = static_cast<qd_unet *>(s->unet);
    if (!u || !u->mode) return QD_OK;
    // on standby no solve of the attempt runs the network, so its next
    // input is not formed; the first solve after the standby reads the last
    // change formed before it (a stale input only weakens that prediction,
    // whose correction is still scaled by the energy-optimal step)
    if (u->mode == 2 && s->net_standby) return QD_OK;
    const LevelDims &d = s->dims[0];
    const UGrid &g = u->g[0];
    QD_CUDA(launch_pdl(true, k_target, dim3(cdv(g.P, 256)), dim3(256), 0, s->stream, (const double *)s->L64[0].u,
                       (const double *)u->d_u_start, d.N, d.K, d.P, (const float *)u->d_scale, u->target32, g,
                       u->stride, (const SolveState *)(u->mode == 2 ? s->d_solve : nullptr)));
    QD_LAUNCH_CHECK(s);
    if (u->mode == 1) {
        QD_TRY(loss_and_grad(u));
        QD_TRY(adam(u));
    }
    // the solved change is the next solve's input channel 4: the buffers
    // trade places (stream order keeps the next writer after every reader)
    float *t = u->d_prev;
    u->d_prev = u->target32;
    u->target32 = t;
    return QD_OK;
}

// where the solution-history guess leaves the boundary data its combination
// implies, so that the network's boundary-change inputs describe what the
// guess still misses (null when no network is in use, and on standby, when
// no solve of the attempt can run the network)
double *warm_start_bc_buffer(qd_solver *s) {
    qd_unet *u = static_cast<qd_unet *>(s->unet);
    if (!u || !u->mode || (u->mode == 2 && s->net_standby)) return nullptr;
    return u->d_bc_old;
}

void warm_start_detach(qd_solver *s) {
    qd_unet *u = static_cast<qd_unet *>(s->unet);
    if (!u) return;
    solve_graph_free(s);
    cudaFree(u->d_u_start);
    u->d_u_start = nullptr;
    u->stream = u->own_stream;
    u->mode = 0;
    s->unet = nullptr;
}

}  // namespace qd

extern "C" {

int qd_unet_create(int nk, int ni, unsigned long long seed, qd_unet **out) {
    if (!out || nk < 17 || ni < 17 || (nk - 1) % 8 || (ni - 1) % 8) {
        set_error("qd_unet_create: grids need (n-1) divisible by 8 and n >= 17");
        return QD_ERR_ARG;
    }
    *out = nullptr;
    qd_unet *u = new qd_unet();
    u->nk = nk; u->ni = ni; u->lr = 1e-3f;
    if (cudaStreamCreateWithFlags(&u->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete u;
        set_error("qd_unet_create: stream creation failed");
        return QD_ERR_CUDA;
    }
    u->stream = u->own_stream;
    const int rc = unet_build(u, seed);
    if (rc != QD_OK) {
        unet_free(u);
        return rc;
    }
    *out = u;
    return QD_OK;
}

void qd_unet_destroy(qd_unet *u) {
    if (u) unet_free(u);
}

long long qd_unet_num_params(const qd_unet *u) {
    if (!u) return -1;
    long long n = 0;
    for (const auto &Ly : u->L) n += 9LL * Ly.cout * Ly.cin + Ly.cout;
    return n;
}

static int params_io(qd_unet *u, float *host, int get, int grads) {
    long long off = 0;
    for (auto &Ly : u->L) {
        const size_t nw = (size_t)9 * Ly.cout * Ly.cin;
        float *w = grads ? Ly.gw : Ly.w32, *b = grads ? Ly.gb : Ly.b32;
        if (get) {
            QD_CUDA(cudaMemcpy(host + off, w, nw * sizeof(float), cudaMemcpyDeviceToHost));
            QD_CUDA(cudaMemcpy(host + off + nw, b, Ly.cout * sizeof(float), cudaMemcpyDeviceToHost));
        } else {
            QD_CUDA(cudaMemcpy(w, host + off, nw * sizeof(float), cudaMemcpyHostToDevice));
            QD_CUDA(cudaMemcpy(b, host + off + nw, Ly.cout * sizeof(float), cudaMemcpyHostToDevice));
            k_weights_bf16<<<cdv((long)nw, 256), 256, 0, u->stream>>>(Ly);
            QD_CUDA(cudaPeekAtLastError());
        }
        off += nw + Ly.cout;
    }
    QD_CUDA(cudaStreamSynchronize(u->stream));
    return QD_OK;
}

int qd_unet_get_params(qd_unet *u, float *host) {
    if (!u || !host) return QD_ERR_ARG;
    return params_io(u, host, 1, 0);
}

int qd_unet_set_params(qd_unet *u, const float *host) {
    if (!u || !host) return QD_ERR_ARG;
    return params_io(u, const_cast<float *>(host), 0, 0);
}

int qd_unet_forward_host(qd_unet *u, const float *x, float *y) {
    if (!u || !x || !y) return QD_ERR_ARG;
    QD_TRY(upload_input(u, x, nullptr));
    QD_TRY(forward(u));
    const UGrid &g = u->g[0];
    float *tmp = nullptr;
    QD_CUDA(cudaMalloc(&tmp, sizeof(float) * (size_t)g.H * g.W));
    k_unpad_f32<<<cdv((long)g.H * g.W, 256), 256, 0, u->stream>>>(u->out32, tmp, g);
    int rc = check_unet_status(u);
    if (rc == QD_OK && cudaMemcpy(y, tmp, sizeof(float) * (size_t)g.H * g.W, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = QD_ERR_CUDA;
    cudaFree(tmp);
    return rc;
}

int qd_unet_loss_grad_host(qd_unet *u, const float *x, const float *target, float *loss, float *grads) {
    if (!u || !x || !target || !loss) return QD_ERR_ARG;
    QD_TRY(upload_input(u, x, target));
    QD_TRY(loss_and_grad(u));
    QD_TRY(check_unet_status(u));
    QD_CUDA(cudaMemcpy(loss, u->d_loss, sizeof(float), cudaMemcpyDeviceToHost));
    if (grads) QD_TRY(params_io(u, grads, 1, 1));
    return QD_OK;
}

int qd_unet_train_step_host(qd_unet *u, const float *x, const float *target, float lr, float *loss) {
    if (!u || !x || !target || !(lr > 0.f)) return QD_ERR_ARG;
    u->lr = lr;
    QD_TRY(upload_input(u, x, target));
    QD_TRY(loss_and_grad(u));
    QD_TRY(adam(u));
    QD_TRY(check_unet_status(u));
    if (loss) QD_CUDA(cudaMemcpy(loss, u->d_loss, sizeof(float), cudaMemcpyDeviceToHost));
    return QD_OK;
}

int qd_solver_warm_start(qd_solver *s, qd_unet *u, int mode, float lr) {
    if (!s || mode < 0 || mode > 2 || (mode && !u) || (mode == 1 && !(lr > 0.f))) {
        set_error("qd_solver_warm_start: bad arguments");
        return QD_ERR_ARG;
    }
    int stride = 1;
    if (u && (u->nk != s->nk || u->ni != s->ni)) {
        if (2 * u->nk - 1 == s->nk && 2 * u->ni - 1 == s->ni) {
            stride = 2;   // the network on the solver's level-1 grid
        } else if (4 * u->nk - 3 == s->nk && 4 * u->ni - 3 == s->ni) {
            stride = 4;   // on its level-2 grid
        } else {
            set_error("qd_solver_warm_start: network grid %dx%d is not the solver's %dx%d grid, nor its level-1 "
                      "or level-2 grid", u->nk, u->ni, s->nk, s->ni);
            return QD_ERR_ARG;
        }
    }
    QD_CUDA(cudaStreamSynchronize(s->stream));
    if (s->unet && s->unet != u) {
        qd_unet *old = static_cast<qd_unet *>(s->unet);
        QD_CUDA(cudaStreamSynchronize(old->stream));
        warm_start_detach(s);
    }
    if (!u || !mode) {
        if (s->unet) warm_start_detach(s);
        return QD_OK;
    }
    QD_CUDA(cudaStreamSynchronize(u->stream));
    if (!u->d_u_start) QD_CUDA(cudaMalloc(&u->d_u_start, sizeof(double) * (size_t)s->dims[0].N * s->dims[0].P));
    if (s->unet != u) QD_CUDA(cudaMemset(u->d_prev, 0, sizeof(float) * (size_t)u->g[0].P));   // a new run
    solve_graph_free(s);     // the solve graph holds the attached network's kernels
    s->net_standby = false;
    u->stream = s->stream;   // the net runs on the solver's stream while attached
    u->stride = stride;
    u->mode = mode;
    u->lr = mode == 1 ? lr : u->lr;
    s->unet = u;
    return QD_OK;
}

// s->net_ratio: >= 1 a fixed ratio; <= 0 the measured rule with a cost of
// -net_ratio V-cycles (solve_begin_dev)
int qd_solver_warm_start_gate(qd_solver *s, double ratio) {
    if (!s || !(ratio == 0.0 || ratio >= 1.0) || !isfinite(ratio)) {
        set_error("qd_solver_warm_start_gate: ratio must be 0 or finite and >= 1");
        return QD_ERR_ARG;
    }
    s->net_ratio = ratio == 0.0 ? -s->net_cost : ratio;
    return QD_OK;
}

int qd_solver_warm_start_cost(qd_solver *s, double cycles) {
    if (!s || !(cycles >= 0.0) || !isfinite(cycles)) {
        set_error("qd_solver_warm_start_cost: the cost must be finite and >= 0 V-cycles");
        return QD_ERR_ARG;
    }
    s->net_cost = cycles;
    if (s->net_ratio <= 0.0) s->net_ratio = -cycles;
    return QD_OK;
}

// the first convolution of the forward pass alone
static int first_conv(qd_unet *u) {
    ULayer &Ly = u->L[0];
    ConvArgs a = conv_args(u, u->g[Ly.lvl], Ly.cin, Ly.cout);
    a.relu = Ly.relu;
    a.bias = Ly.b32;
    a.out = Ly.out->p;
    return conv_dispatch(u, Ly.m_in, Ly.rows_fwd ? &Ly.m_in_rows : nullptr, Ly.m_w, a);
}

int qd_unet_time(qd_unet *u, int what, int reps, double *us, double *flops) {
    if (!u || what < 0 || what > 2 || reps < 1 || !us) return QD_ERR_ARG;
    double f = 0.0;
    for (const auto &Ly : u->L) {
        const UGrid &g = u->g[Ly.lvl];
        const double conv = 2.0 * 9.0 * Ly.cin * Ly.cout * (double)g.H * g.W;
        if (what == 2) {
            f = conv;
            break;
        }
        f += conv * (what ? (Ly.gin ? 3.0 : 2.0) : 1.0);
    }
    if (flops) *flops = f;
    cudaEvent_t e0, e1;
    QD_CUDA(cudaEventCreate(&e0));
    QD_CUDA(cudaEventCreate(&e1));
    int rc = cudaEventRecord(e0, u->stream) == cudaSuccess ? QD_OK : QD_ERR_CUDA;
    for (int i = 0; i < reps && rc == QD_OK; i++)
        rc = what == 2 ? first_conv(u) : (what ? loss_and_grad(u) : forward(u));
    float ms = 0.f;
    if (rc == QD_OK && (cudaEventRecord(e1, u->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
        rc = QD_ERR_CUDA;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == QD_OK) rc = check_unet_status(u);
    if (rc == QD_OK) *us = 1e3 * ms / reps;
    return rc;
}

int qd_unet_stats(qd_unet *u, long long *train_steps, float *last_loss) {
    if (!u) return QD_ERR_ARG;
    if (train_steps) *train_steps = u->steps;
    if (last_loss) {
        QD_CUDA(cudaStreamSynchronize(u->stream));
        QD_CUDA(cudaMemcpy(last_loss, u->d_loss, sizeof(float), cudaMemcpyDeviceToHost));
    }
    return QD_OK;
}

}  // extern "C"
