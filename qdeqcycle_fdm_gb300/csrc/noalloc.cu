// noalloc.cu -- qd_residual_norm_noalloc: the level-0 residual norm of
// multigrid() (calcuDelta + the L2 norm, odeSolver.cpp:693-694) on arrays the
// caller owns, with no device allocation at all.
//
// Who needs it: a caller that cannot allocate device memory at the moment it
// asks for a norm -- a host framework that owns every device byte through
// its own allocator or a budget fixed at start-up, or an embedding where a
// cudaMalloc would synchronise the device in the middle of its own work.
// Such a caller holds u and the face moduli already and only needs the
// number.  The block partial sums that the solver keeps in its own scratch
// buffer live here in a file-scope device array instead: every GPU that
// loads the library holds it until the process exits.
#include <math.h>

#include <mutex>

#include "qdeq_internal.cuh"

namespace qd {
namespace {

constexpr int NA_BX = 32, NA_BY = 8;           // the solver's residual block shape
// The largest grid is 4097 x 4097 nodes (rows and columns each checked):
// ceil(4097 / 32) = 129 block columns x ceil(4097 / 8) = 513 block rows =
// 66,177 partial sums, and one more slot for the total: 66,178 doubles =
// 529,424 bytes (517 KB) per GPU.
constexpr int NOALLOC_MAX_N = 4097;
constexpr int NOALLOC_MAX_PARTIALS = ((NOALLOC_MAX_N + NA_BX - 1) / NA_BX) * ((NOALLOC_MAX_N + NA_BY - 1) / NA_BY);
static_assert(NOALLOC_MAX_PARTIALS == 66177, "129 x 513 blocks");

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_MAX_PARTIALS + 1];

std::mutex g_mutex;
double *g_scratch_dev[64] = {};                 // device address of the array, per device

__device__ double na_block_sum(double v) {
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
    return v;
}

// r = 0 - A u on the interior columns (the same expression as the solver's
// level-0 residual); one partial sum of r^2 per block
__global__ void __launch_bounds__(NA_BX *NA_BY)
    k_noalloc_partials(const double *u, const double *cx, const double *cz, int N, int K, int P,
                       double inv_h2, double *partial) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    double sq = 0.0;
    if (j < N && k >= 1 && k <= K - 2) {
        const long c = (long)j * P + k;
        const long up = (j == 0) ? P : -(long)P;
        const long dn = (j == N - 1) ? -(long)P : P;
        const double cW = cx[c - 1], cE = cx[c], cN = cz[c], cS = cz[c + P];
        const double lap = cW * u[c - 1] + cE * u[c + 1] + cN * u[c + up] + cS * u[c + dn] -
                           (((cW + cE) + cN) + cS) * u[c];
        const double res = 0.0 - lap * inv_h2;
        sq = res * res;
    }
    sq = na_block_sum(sq);
    if (threadIdx.x == 0 && threadIdx.y == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = sq;
}

__global__ void k_noalloc_total(const double *partial, int n, double *out) {
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += partial[i];
    v = na_block_sum(v);
    if (threadIdx.x == 0) *out = v;
}

// The array's device address for the current device, looked up once per
// device (host code cannot use the symbol itself as a device pointer) and
// kept for the life of the process.  A cudaDeviceReset reloads the module,
// which may move the array, so calls after a reset of a device that already
// ran this entry point are not supported.
int scratch_for_current_device(double **out) {
    int dev = 0;
    QD_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("qd_residual_norm_noalloc: device ordinal %d out of range", dev);
        return QD_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_dev[dev]) {
        void *p = nullptr;
        QD_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch_dev[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_dev[dev];
    return QD_OK;
}

}  // namespace
}  // namespace qd

extern "C" int qd_residual_norm_noalloc(const double *u, const double *cx, const double *cz, int nk,
                                        int ni, int pitch, double dh, void *stream, double *rnorm) {
    using namespace qd;
    if (!u || !cx || !cz || !rnorm || nk < 3 || ni < 3 || pitch < ni || !(dh > 0.0)) {
        set_error("qd_residual_norm_noalloc: bad arguments (nk=%d ni=%d pitch=%d)", nk, ni, pitch);
        return QD_ERR_ARG;
    }
    if (nk > NOALLOC_MAX_N || ni > NOALLOC_MAX_N) {
        set_error("qd_residual_norm_noalloc: a %d x %d grid is larger than the static scratch "
                  "allows (at most %d rows and %d columns)", nk, ni, NOALLOC_MAX_N, NOALLOC_MAX_N);
        return QD_ERR_ARG;
    }
    const int gx = (ni + NA_BX - 1) / NA_BX, gy = (nk + NA_BY - 1) / NA_BY;
    const long nb = (long)gx * gy;     // <= NOALLOC_MAX_PARTIALS by the check above
    double *scratch = nullptr;
    QD_TRY(scratch_for_current_device(&scratch));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_noalloc_partials<<<dim3(gx, gy), dim3(NA_BX, NA_BY), 0, st>>>(u, cx, cz, nk, ni, pitch,
                                                                    1.0 / (dh * dh), scratch);
    QD_CUDA(cudaGetLastError());
    // every slot the total reads was just written, so nothing needs clearing
    k_noalloc_total<<<1, 1024, 0, st>>>(scratch, (int)nb, scratch + NOALLOC_MAX_PARTIALS);
    QD_CUDA(cudaGetLastError());
    double sum = 0.0;
    QD_CUDA(cudaMemcpyAsync(&sum, scratch + NOALLOC_MAX_PARTIALS, sizeof(double),
                            cudaMemcpyDeviceToHost, st));
    QD_CUDA(cudaStreamSynchronize(st));
    *rnorm = sqrt(sum);
    return QD_OK;
}
