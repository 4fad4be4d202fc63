// io.cu -- files around the RK43 run: the reference's initial-displacement
// input (odeSolver.cpp:96-128), its snapshot records (odeSolver.cpp:1442-1456
// and :1638-1652) written from the device state without stalling the
// solver, and a checkpoint / restart file that resumes a run bit for bit.
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "qdeq_internal.cuh"

namespace qd {

// One snapshot in flight per solver: device -> pinned copies enqueued on the
// solver's stream, then a host thread waits for them and writes the file.
struct SnapshotJob {
    std::thread th;
    cudaEvent_t ev = nullptr;
    double *pin = nullptr;       // V, Slip, Ts, psi, Tn, a, b (nz each) + u (N x K)
    size_t pin_elems = 0;
    int rc = QD_OK;
    char err[256] = "";
};

static SnapshotJob *job_of(qd_solver *s) {
    if (!s->snapshot) s->snapshot = new SnapshotJob();
    return static_cast<SnapshotJob *>(s->snapshot);
}

// ghost fill of extend_crew (odeSolver.cpp:612-650) on a host array
static void extend_crew_fill(int ni, int nk, double *U) {
    const int nx = ni + 2, nz = nk + 2;
    for (int k = 0; k < nz; k++) {
        double *row = U + (long)k * nx;
        row[0] = 2.0 * row[1] - row[2];
        row[ni + 1] = 2.0 * row[ni] - row[ni - 1];
    }
    for (int i = 0; i < nx; i++) {
        U[i] = U[i + 2L * nx];
        U[i + (long)(nk + 1) * nx] = U[i + (long)(nk - 1) * nx];
    }
}

static int write_all(FILE *fp, const void *p, size_t bytes) {
    return fwrite(p, 1, bytes, fp) == bytes ? QD_OK : QD_ERR_ARG;
}

}  // namespace qd

using namespace qd;

extern "C" {

int qd_snapshot_wait(qd_solver *s) {
    if (!s) return QD_ERR_ARG;
    SnapshotJob *j = static_cast<SnapshotJob *>(s->snapshot);
    if (!j || !j->th.joinable()) return QD_OK;
    j->th.join();
    if (j->rc != QD_OK) set_error("%s", j->err);
    return j->rc;
}

int qd_snapshot(qd_solver *s, const char *path, int full, int async) {
    if (!s || !path || !s->fault_ready) {
        set_error("qd_snapshot: bad arguments or fault state not set up");
        return QD_ERR_ARG;
    }
    QD_TRY(qd_snapshot_wait(s));
    SnapshotJob *j = job_of(s);
    const int nz = s->nz, N = s->dims[0].N, K = s->dims[0].K;
    const size_t need = 7 * (size_t)nz + (size_t)N * K;
    if (j->pin_elems < need) {
        cudaFreeHost(j->pin);
        j->pin = nullptr;
        QD_CUDA(cudaMallocHost(&j->pin, need * sizeof(double)));
        j->pin_elems = need;
    }
    if (!j->ev) QD_CUDA(cudaEventCreateWithFlags(&j->ev, cudaEventDisableTiming));
    double *h = j->pin;
    const double *src[7] = {s->F.fV[1], s->F.Slip, s->F.Ts, s->F.psi, s->F.Tn, s->F.a, s->F.b};
    for (int i = 0; i < 7; i++)
        QD_CUDA(cudaMemcpyAsync(h + (size_t)i * nz, src[i], nz * sizeof(double), cudaMemcpyDeviceToHost,
                                s->stream));
    if (full)
        QD_CUDA(cudaMemcpy2DAsync(h + 7 * (size_t)nz, K * sizeof(double), s->L64[0].u,
                                  s->dims[0].P * sizeof(double), K * sizeof(double), N,
                                  cudaMemcpyDeviceToHost, s->stream));
    QD_CUDA(cudaEventRecord(j->ev, s->stream));
    const double t = s->t, dt = s->dt;
    const int ni = s->ni, nk = s->nk;
    const std::string file(path);
    j->rc = QD_OK;
    j->err[0] = 0;
    auto work = [j, file, t, dt, nz, ni, nk, full]() {
        if (cudaEventSynchronize(j->ev) != cudaSuccess) {
            j->rc = QD_ERR_CUDA;
            snprintf(j->err, sizeof(j->err), "qd_snapshot: device copies failed");
            return;
        }
        const double *h = j->pin;
        std::vector<double> U;
        if (full) {
            const int nx = ni + 2;
            U.assign((size_t)nx * (nk + 2), 0.0);
            for (int k = 0; k < nk; k++)
                memcpy(&U[(size_t)(k + 1) * nx + 1], h + 7 * (size_t)nz + (size_t)k * ni, ni * sizeof(double));
            extend_crew_fill(ni, nk, U.data());
        }
        FILE *fp = fopen(file.c_str(), "wb");
        int rc = fp ? QD_OK : QD_ERR_ARG;
        const size_t b = nz * sizeof(double);
        // t, V, Slip, Ts, psi [, U, Tn, a, b], dt
        if (rc == QD_OK) rc = write_all(fp, &t, sizeof(double));
        for (int i = 0; i < 4 && rc == QD_OK; i++) rc = write_all(fp, h + (size_t)i * nz, b);
        if (full) {
            if (rc == QD_OK) rc = write_all(fp, U.data(), U.size() * sizeof(double));
            for (int i = 4; i < 7 && rc == QD_OK; i++) rc = write_all(fp, h + (size_t)i * nz, b);
        }
        if (rc == QD_OK) rc = write_all(fp, &dt, sizeof(double));
        if (fp && fclose(fp) != 0) rc = QD_ERR_ARG;
        if (rc != QD_OK) {
            j->rc = rc;
            snprintf(j->err, sizeof(j->err), "qd_snapshot: cannot write %s", file.c_str());
        }
    };
    if (async) {
        j->th = std::thread(work);
        return QD_OK;
    }
    work();
    if (j->rc != QD_OK) set_error("%s", j->err);
    return j->rc;
}

// Checkpoint file, little-endian:
//   char[8] "QDEQCKP1"; int32 ni, nk, it, maxNumSteps;
//   double t, dt, errA0, errA1, tmax, ini_dt, mindt, maxdt, totTol;
//   double Slip, psi, V, Ts, dpsi [nz each]; double u [nk][ni]
static const char kMagic[8] = {'Q', 'D', 'E', 'Q', 'C', 'K', 'P', '1'};

int qd_checkpoint_save(qd_solver *s, const char *path) {
    if (!s || !path || !s->started) {
        set_error("qd_checkpoint_save: bad arguments or RK43 not started");
        return QD_ERR_ARG;
    }
    const int nz = s->nz, N = s->dims[0].N, K = s->dims[0].K;
    std::vector<double> v(5 * (size_t)nz + (size_t)N * K);
    const double *src[5] = {s->F.Slip, s->F.psi, s->F.fV[1], s->F.Ts, s->F.fdpsi[1]};
    for (int i = 0; i < 5; i++)
        QD_CUDA(cudaMemcpyAsync(v.data() + (size_t)i * nz, src[i], nz * sizeof(double), cudaMemcpyDeviceToHost,
                                s->stream));
    QD_CUDA(cudaMemcpy2DAsync(v.data() + 5 * (size_t)nz, K * sizeof(double), s->L64[0].u,
                              s->dims[0].P * sizeof(double), K * sizeof(double), N, cudaMemcpyDeviceToHost,
                              s->stream));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    FILE *fp = fopen(path, "wb");
    if (!fp) {
        set_error("qd_checkpoint_save: cannot open %s", path);
        return QD_ERR_ARG;
    }
    const int hdr[4] = {s->ni, s->nk, s->it, s->P.maxNumSteps};
    const double sc[9] = {s->t, s->dt, s->errA[0], s->errA[1], s->P.tmax, s->P.ini_dt, s->P.mindt,
                          s->P.maxdt, s->P.totTol};
    int rc = write_all(fp, kMagic, 8);
    if (rc == QD_OK) rc = write_all(fp, hdr, sizeof(hdr));
    if (rc == QD_OK) rc = write_all(fp, sc, sizeof(sc));
    if (rc == QD_OK) rc = write_all(fp, v.data(), v.size() * sizeof(double));
    if (fclose(fp) != 0) rc = QD_ERR_ARG;
    if (rc != QD_OK) set_error("qd_checkpoint_save: cannot write %s", path);
    return rc;
}

int qd_checkpoint_load(qd_solver *s, const char *path) {
    if (!s || !path || !s->fault_ready) {
        set_error("qd_checkpoint_load: bad arguments or fault state not set up");
        return QD_ERR_ARG;
    }
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        set_error("qd_checkpoint_load: cannot open %s", path);
        return QD_ERR_ARG;
    }
    char magic[8];
    int hdr[4];
    double sc[9];
    const int nz = s->nz, N = s->dims[0].N, K = s->dims[0].K;
    std::vector<double> v(5 * (size_t)nz + (size_t)N * K);
    bool ok = fread(magic, 1, 8, fp) == 8 && memcmp(magic, kMagic, 8) == 0 &&
              fread(hdr, sizeof(int), 4, fp) == 4 && hdr[0] == s->ni && hdr[1] == s->nk &&
              fread(sc, sizeof(double), 9, fp) == 9 && fread(v.data(), sizeof(double), v.size(), fp) == v.size();
    fclose(fp);
    if (!ok) {
        set_error("qd_checkpoint_load: %s is not a checkpoint of a %d x %d grid", path, s->nk, s->ni);
        return QD_ERR_ARG;
    }
    double *dst[5] = {s->F.Slip, s->F.psi, s->F.fV[1], s->F.Ts, s->F.fdpsi[1]};
    for (int i = 0; i < 5; i++)
        QD_CUDA(cudaMemcpyAsync(dst[i], v.data() + (size_t)i * nz, nz * sizeof(double), cudaMemcpyHostToDevice,
                                s->stream));
    QD_CUDA(cudaMemcpy2DAsync(s->L64[0].u, s->dims[0].P * sizeof(double), v.data() + 5 * (size_t)nz,
                              K * sizeof(double), K * sizeof(double), N, cudaMemcpyHostToDevice, s->stream));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    s->it = hdr[2];
    s->P.maxNumSteps = hdr[3];
    s->t = sc[0]; s->dt = sc[1]; s->errA[0] = sc[2]; s->errA[1] = sc[3];
    s->P.tmax = sc[4]; s->P.ini_dt = sc[5]; s->P.mindt = sc[6]; s->P.maxdt = sc[7]; s->P.totTol = sc[8];
    s->started = 1;
    history_reset(s);     // the file holds no solution history: it restarts here
    return QD_OK;
}

int qd_load_initial_u(const char *path, int ni, int nk, double *U) {
    if (!path || !U || ni < 1 || nk < 1) {
        set_error("qd_load_initial_u: bad arguments");
        return QD_ERR_ARG;
    }
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        set_error("qd_load_initial_u: cannot open %s", path);
        return QD_ERR_ARG;
    }
    std::vector<double> u0((size_t)ni * nk);
    const size_t got = fread(u0.data(), sizeof(double), u0.size(), fp);
    fclose(fp);
    if (got != u0.size()) {
        set_error("qd_load_initial_u: %s holds %zu of the %zu values of a %d x %d grid", path, got,
                  u0.size(), nk, ni);
        return QD_ERR_ARG;
    }
    const int nx = ni + 2;
    for (int k = 0; k < nk; k++)
        for (int i = 0; i < ni; i++) U[(size_t)(k + 1) * nx + (i + 1)] = u0[(size_t)k * ni + i];
    return QD_OK;
}

int qd_save_initial_u(const char *path, int ni, int nk, const double *U) {
    if (!path || !U || ni < 1 || nk < 1) {
        set_error("qd_save_initial_u: bad arguments");
        return QD_ERR_ARG;
    }
    FILE *fp = fopen(path, "wb");
    if (!fp) {
        set_error("qd_save_initial_u: cannot open %s", path);
        return QD_ERR_ARG;
    }
    const int nx = ni + 2;
    int rc = QD_OK;
    for (int k = 0; k < nk && rc == QD_OK; k++) rc = write_all(fp, U + (size_t)(k + 1) * nx + 1, ni * sizeof(double));
    if (fclose(fp) != 0) rc = QD_ERR_ARG;
    if (rc != QD_OK) set_error("qd_save_initial_u: cannot write %s", path);
    return rc;
}

}  // extern "C"

namespace qd {
void snapshot_free(qd_solver *s) {
    SnapshotJob *j = static_cast<SnapshotJob *>(s->snapshot);
    if (!j) return;
    if (j->th.joinable()) j->th.join();
    if (j->ev) cudaEventDestroy(j->ev);
    cudaFreeHost(j->pin);
    delete j;
    s->snapshot = nullptr;
}
}  // namespace qd
