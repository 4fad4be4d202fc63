// autotune.cu -- picks the multigrid's smoother schedule and tile shapes by
// measurement on the solver's own problem.
//
// A candidate is a smoother schedule (nu_pre, nu_post red+black sweeps per
// level) and a pair of staged tile box widths for the descending (k_down)
// and ascending (k_up) tile kernels; the box width sets the tile width and,
// through the shared-memory budget of two CTAs per SM, the tile height and
// the halo overhead.  Each candidate is timed on `reps` solves to the
// solver's tolerance, with CUDA events around the solve graph on the
// solver's stream; the fastest is kept.  The solves are those the run
// makes: with a solution history of at least three solutions, the last
// stored solve replayed from the history guess of the solutions before it
// (history_replay_guess: a starting residual like the run's own, which a
// solve clears in about one V-cycle, so per-cycle cost ranks the
// candidates), as long as that solve takes a V-cycle with the starting
// settings (one that starts within the tolerance times no cycle and ranks
// nothing); otherwise the solver's current boundary data from a zero
// interior (the guess-independent reference point of the relative
// tolerance, several V-cycles, where the convergence rate weighs in).  An
// attached network is left out of the timed solves (the tuner
// times the multigrid).  u and the solve counters are restored afterwards,
// so tuning leaves the simulation state as it found it.  The reference has no tuner: its
// schedule is fixed at V(32,32) on 6 levels (odeSolver.cpp:2-4).
#include <math.h>

#include <vector>

#include "qdeq_internal.cuh"

namespace qd {

namespace {

struct Candidate {
    int nu_pre, nu_post, box_up, box_down;
};

struct Saved {
    double *u = nullptr;
    SolveState st{};
};

// zero the interior columns 1..K-2 of u (the boundary columns keep the data)
int zero_interior(qd_solver *s) {
    const LevelDims &d = s->dims[0];
    QD_CUDA(cudaMemset2DAsync(s->L64[0].u + 1, (size_t)d.P * sizeof(double), 0, (size_t)(d.K - 2) * sizeof(double),
                              d.N, s->stream));
    return QD_OK;
}

int restore_u(qd_solver *s, const Saved &sv) {
    const LevelDims &d = s->dims[0];
    QD_CUDA(cudaMemcpyAsync(s->L64[0].u, sv.u, sizeof(double) * (size_t)d.N * d.P, cudaMemcpyDeviceToDevice,
                            s->stream));
    return QD_OK;
}

// the starting field of a timed solve (see the head of the file)
int start_field(qd_solver *s, const Saved &sv, bool replay) {
    if (replay) return history_replay_guess(s);
    QD_TRY(restore_u(s, sv));
    return zero_interior(s);
}

// mean microseconds of one solve with the solver's current settings; QD_OK
// with *us = +inf when the setting is not usable
int time_solves(qd_solver *s, const Saved &sv, bool replay, int reps, cudaEvent_t e0, cudaEvent_t e1,
                double *us, int *cycles) {
    *us = INFINITY;
    *cycles = -1;
    // one untimed solve: builds the graph and checks that the setting converges
    QD_TRY(start_field(s, sv, replay));
    int cyc = 0;
    double rn = 0.0;
    int rc = mg_solve(s, &cyc, &rn, nullptr);
    if (rc == QD_ERR_NOT_CONVERGED || rc == QD_ERR_ARG) return QD_OK;   // skip this candidate
    QD_TRY(rc);
    double total = 0.0;
    for (int r = 0; r < reps; r++) {
        QD_TRY(start_field(s, sv, replay));
        QD_CUDA(cudaEventRecord(e0, s->stream));
        QD_TRY(mg_solve_async(s));
        QD_CUDA(cudaEventRecord(e1, s->stream));
        QD_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        QD_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        total += ms;
    }
    SolveState st;
    QD_TRY(solve_state_read(s, &st));
    if (st.flag) return QD_OK;
    *us = 1e3 * total / reps;
    *cycles = cyc;
    return QD_OK;
}

int apply(qd_solver *s, const Candidate &c) {
    s->opt.nu_pre = c.nu_pre;
    s->opt.nu_post = c.nu_post;
    return tiles_set(s, c.box_up, c.box_down);
}

}  // namespace

int autotune(qd_solver *s, int reps, qd_tuning *out) {
    const LevelDims &d = s->dims[0];
    const Candidate initial{s->opt.nu_pre, s->opt.nu_post, s->box_up, s->box_down};
    std::vector<Candidate> cands;
    cands.push_back(initial);
    const int sched[][2] = {{1, 1}, {2, 2}, {3, 3}, {4, 4}, {1, 2}, {2, 1}, {2, 3}, {3, 2}};
    const int boxes[] = {64, 96, 128};
    int def_up = 0, def_down = 0;
    tiles_default_level0(s, &def_up, &def_down);
    const int eff_up = initial.box_up ? initial.box_up : def_up;
    const int eff_down = initial.box_down ? initial.box_down : def_down;
    for (const auto &sc : sched)
        for (int bu : boxes)
            for (int bd : boxes) {
                const Candidate c{sc[0], sc[1], bu, bd};
                const bool same = c.nu_pre == initial.nu_pre && c.nu_post == initial.nu_post &&
                                  bu == eff_up && bd == eff_down;
                if (!same) cands.push_back(c);
            }

    Saved sv;
    s->net_paused = true;
    struct Resume {
        qd_solver *s;
        ~Resume() { s->net_paused = false; }
    } resume{s};
    QD_CUDA(cudaMalloc(&sv.u, sizeof(double) * (size_t)d.N * d.P));
    QD_CUDA(cudaMemcpyAsync(sv.u, s->L64[0].u, sizeof(double) * (size_t)d.N * d.P, cudaMemcpyDeviceToDevice,
                            s->stream));
    int rc = solve_state_read(s, &sv.st);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (rc == QD_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) {
        set_error("autotune: event creation failed");
        rc = QD_ERR_CUDA;
    }
    // replay the last stored solve where the history holds one and the
    // replayed solve takes a cycle
    bool replay = rc == QD_OK && history_replay_guess(s) == QD_OK;
    if (replay) {
        int cyc = 0;
        double rn = 0.0;
        const int r = mg_solve(s, &cyc, &rn, nullptr);
        if (r == QD_OK) replay = cyc > 0;
        else if (r == QD_ERR_NOT_CONVERGED) replay = false;
        else rc = r;
    }
    double best_us = INFINITY, init_us = INFINITY;
    int best_cyc = -1, init_cyc = -1, timed = 0;
    Candidate best = initial;
    for (size_t i = 0; i < cands.size() && rc == QD_OK; i++) {
        rc = apply(s, cands[i]);
        if (rc != QD_OK) break;
        double us = INFINITY;
        int cyc = -1;
        rc = time_solves(s, sv, replay, reps, e0, e1, &us, &cyc);
        if (rc != QD_OK) break;
        if (isfinite(us)) timed++;
        if (i == 0) {
            init_us = us;
            init_cyc = cyc;
        }
        if (us < best_us) {
            best_us = us;
            best_cyc = cyc;
            best = cands[i];
        }
    }
    // the winner, and the state as it was
    if (rc == QD_OK) rc = apply(s, isfinite(best_us) ? best : initial);
    if (rc == QD_OK) rc = restore_u(s, sv);
    if (rc == QD_OK) {
        if (cudaMemcpyAsync(s->d_solve, &sv.st, sizeof(SolveState), cudaMemcpyHostToDevice, s->stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(s->stream) != cudaSuccess) {
            set_error("autotune: restoring the solve state failed");
            rc = QD_ERR_CUDA;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sv.u);
    if (rc != QD_OK) return rc;
    if (out) {
        out->nu_pre = s->opt.nu_pre;
        out->nu_post = s->opt.nu_post;
        out->box_up = s->box_up ? s->box_up : 64;
        out->box_down = s->box_down ? s->box_down : 64;
        out->us_best = best_us;
        out->us_initial = init_us;
        out->cycles_best = best_cyc;
        out->cycles_initial = init_cyc;
        out->candidates = timed;
        out->replayed = replay ? 1 : 0;
    }
    return QD_OK;
}

}  // namespace qd

using namespace qd;

extern "C" {

int qd_autotune(qd_solver *s, int reps, qd_tuning *out) {
    if (!s || reps < 1) return QD_ERR_ARG;
    return autotune(s, reps, out);
}

int qd_set_tiles(qd_solver *s, int box_up, int box_down) {
    if (!s) return QD_ERR_ARG;
    return tiles_set(s, box_up, box_down);
}

}  // extern "C"
