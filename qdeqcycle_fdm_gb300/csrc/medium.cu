// medium.cu -- SetMedium's face-modulus homogenisation on the GPU
// (odeSolver.cpp:337-589).
//
// Each cell face gets the harmonic mean of 400 samples of a Lagrange
// interpolant through the 3x4 (x-faces) or 4x3 (z-faces) surrounding nodes
// of mu_half.  The 400 sample abscissae are the same for every face, so the
// Lagrange basis values are computed once on the host (with the reference's
// product loop, odeSolver.cpp:140-187) and broadcast from constant memory;
// each thread then does 400 x 12 multiply-adds and 400 reciprocals for one
// face, summing in the reference's order (j outer, i inner, :190-197).
// The reference leaves mu_matrix[1][1] unset for x-faces (:434-436); here it
// is the node that slot stands for, mu_half[index3 + 2].
#include <cstring>
#include <vector>

#include "qdeq_internal.cuh"

namespace qd {

static constexpr int NGRID = 10;
static constexpr int NSAMP = (2 * NGRID) * (2 * NGRID);

struct MediumBasis {
    double LxA[NSAMP][3], LyA[NSAMP][4];   // x-face stencil: 3 rows x 4 columns
    double LxB[NSAMP][4], LyB[NSAMP][3];   // z-face stencil: 4 rows x 3 columns
};
__constant__ MediumBasis c_basis;

static void lagrange_basis(const double *x, int n, double xi, double *L) {
    double xt[8], xb[8];
    for (int k = 0; k < n; k++) L[k] = 1.0;
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < n; k++) xb[k] = x[i] - x[k];
        xb[i] = 1.0;
        for (int k = 0; k < n; k++) xt[k] = xi - x[k];
        xt[i] = 1.0;
        for (int j = 0; j < n; j++) L[i] = L[i] * xt[j] / xb[j];
    }
}

// x-face between ghosted node columns i-1 and i on node row k
// (k = 1..nk, i = 2..ni), odeSolver.cpp:421-461
__global__ void k_xfaces(const double *__restrict__ mh, long W, int ni, int nk, double *me) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
    const int k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > ni || k > nk) return;
    double z[3][4];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) z[r][c] = mh[(i - 2) * 2 + 2 * c + (long)((k - 1 + r) * 2) * W];
    double mu0 = 0.0;
    for (int s = 0; s < NSAMP; s++) {
        double zi = 0.0;
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int r = 0; r < 3; r++) zi = zi + c_basis.LxA[s][r] * c_basis.LyA[s][j] * z[r][j];
        mu0 = mu0 + 1.0 / zi;
    }
    me[(i * 2 - 1) + (long)(k * 2) * W] = NSAMP / mu0;
}

// z-face between ghosted node rows k-1 and k at node column i
// (k = 1..nk+1, i = 2..ni-1); rows clamp to the ghost rows at both ends,
// which is the reference's mirrored boundary faces (:464-589)
__global__ void k_zfaces(const double *__restrict__ mh, long W, int ni, int nk, double *me) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
    const int k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > ni - 1 || k > nk + 1) return;
    double z[4][3];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        int row = k - 2 + r;
        row = row < 0 ? 0 : (row > nk + 1 ? nk + 1 : row);
#pragma unroll
        for (int c = 0; c < 3; c++) z[r][c] = mh[(i - 1) * 2 + 2 * c + (long)(row * 2) * W];
    }
    double mu0 = 0.0;
    for (int s = 0; s < NSAMP; s++) {
        double zi = 0.0;
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int r = 0; r < 4; r++) zi = zi + c_basis.LxB[s][r] * c_basis.LyB[s][j] * z[r][j];
        mu0 = mu0 + 1.0 / zi;
    }
    me[i * 2 + (long)(k * 2 - 1) * W] = NSAMP / mu0;
}

int set_medium_gpu(int ni, int nk, const double *mu_node, double *mu_equi) {
    if (ni < 4 || nk < 4 || !mu_node || !mu_equi) {
        set_error("qd_set_medium: bad arguments (ni=%d nk=%d)", ni, nk);
        return QD_ERR_ARG;
    }
    const int nx = ni + 2, nz = nk + 2;
    const int ni1 = 2, ni2 = ni + 1, nk1 = 2, nk2 = nk + 1;
    const long W = 2L * nx - 1;
    const size_t n2 = (size_t)(2 * nx - 1) * (2 * nz - 1);
    std::vector<double> mh(n2, 0.0), me(n2, 0.0);
    // node values and mirrored edges, :337-376
    for (int k = nk1 - 1; k < nk2; k++)
        for (int i = ni1 - 1; i < ni2; i++) {
            const long id = i * 2 + (long)(k * 2) * W;
            mh[id] = me[id] = mu_node[i + (long)k * nx];
        }
    for (int i = ni1 - 1; i < ni2; i++) {
        mh[i * 2] = me[i * 2] = mh[i * 2 + (long)((nk1 - 1) * 2) * W];
        const long top = i * 2 + (long)((nz - 1) * 2) * W;
        mh[top] = me[top] = mh[i * 2 + (long)((nk2 - 1) * 2) * W];
    }
    for (int k = 0; k < nz; k++) {
        const long row = (long)(k * 2) * W;
        mh[row] = me[row] = mh[(ni1 - 1) * 2 + row];
        mh[(nx - 1) * 2 + row] = me[(nx - 1) * 2 + row] = mh[(ni2 - 1) * 2 + row];
    }
    // arithmetic midpoints, :381-404
    for (int k = 0; k < nz; k++)
        for (int i = ni1 - 1; i < ni2 - 1; i++) {
            const long row = (long)(k * 2) * W;
            mh[(i * 2 + 1) + row] = 0.50 * (mh[i * 2 + row] + mh[(i + 1) * 2 + row]);
        }
    for (int i = ni1 - 1; i < ni2; i++)
        for (int k = 0; k < nz - 1; k++)
            mh[i * 2 + (long)(k * 2 + 1) * W] =
                0.50 * (mh[i * 2 + (long)(k * 2) * W] + mh[i * 2 + (long)((k + 1) * 2) * W]);

    static MediumBasis hb;
    static bool hb_ready = false;
    if (!hb_ready) {
        const double xA[3] = {-1.0, 0.0, 1.0}, yA[4] = {-1.5, -0.5, 0.5, 1.5};
        const double xB[4] = {-1.5, -0.5, 0.5, 1.5}, yB[3] = {-1.0, 0.0, 1.0};
        int s = 0;
        for (int mj = -NGRID; mj <= NGRID; mj++) {
            if (mj == 0) continue;
            for (int mi = -NGRID; mi <= NGRID; mi++) {
                if (mi == 0) continue;
                const double MI = mi / ((NGRID + 1.0) * 2.0), MJ = mj / ((NGRID + 1.0) * 2.0);
                double L[4];
                lagrange_basis(xA, 3, MI, L); memcpy(hb.LxA[s], L, sizeof(hb.LxA[s]));
                lagrange_basis(yA, 4, MJ, L); memcpy(hb.LyA[s], L, sizeof(hb.LyA[s]));
                lagrange_basis(xB, 4, MI, L); memcpy(hb.LxB[s], L, sizeof(hb.LxB[s]));
                lagrange_basis(yB, 3, MJ, L); memcpy(hb.LyB[s], L, sizeof(hb.LyB[s]));
                s++;
            }
        }
        hb_ready = true;
    }
    QD_CUDA(cudaMemcpyToSymbol(c_basis, &hb, sizeof(hb)));
    double *d_mh = nullptr, *d_me = nullptr;
    QD_CUDA(cudaMalloc(&d_mh, n2 * sizeof(double)));
    QD_CUDA(cudaMalloc(&d_me, n2 * sizeof(double)));
    QD_CUDA(cudaMemcpy(d_mh, mh.data(), n2 * sizeof(double), cudaMemcpyHostToDevice));
    QD_CUDA(cudaMemcpy(d_me, me.data(), n2 * sizeof(double), cudaMemcpyHostToDevice));
    dim3 blk(32, 4);
    k_xfaces<<<dim3((ni - 1 + 31) / 32, (nk + 3) / 4), blk>>>(d_mh, W, ni, nk, d_me);
    k_zfaces<<<dim3((ni - 2 + 31) / 32, (nk + 1 + 3) / 4), blk>>>(d_mh, W, ni, nk, d_me);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(mu_equi, d_me, n2 * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(d_mh);
    cudaFree(d_me);
    if (e != cudaSuccess) {
        set_error("qd_set_medium: %s", cudaGetErrorString(e));
        return QD_ERR_CUDA;
    }
    return QD_OK;
}

}  // namespace qd
