// mg_graph.cu -- multigrid() (odeSolver.cpp:652-720) as one CUDA graph.
//
// The reference reads the residual norm back to the host after every
// V-cycle (a blocking cublasDnrm2, :694,700).  Here the whole solve is one
// graph launch:
//
//   prologue   [||r0|| for the relative tolerance] -> ||r|| of the guess
//              -> k_solve_begin: threshold, first "continue?" decision
//   [IF        with a network in prediction mode attached, and only when
//              the guess misses the tolerance by more than the gate (one
//              V-cycle's measured reduction by default): the network's
//              correction of the guess, then the prologue again on the
//              corrected one]
//   WHILE      body: one V-cycle -> ||r|| -> k_solve_check: next decision
//
// In mixed precision the prologue and the body's check are folded into the
// last block of the level-0 residual's reduction (one kernel each).
//
// The loop condition is a graph conditional handle that the check kernels
// set on the device (cudaGraphSetConditional), so no host round trip
// happens inside a solve.  The loop stops when ||r|| <= threshold, when the
// cycle cap is reached or when the norm is not finite; the last two leave a
// flag the host reads with the next result it fetches.  The graph is built
// from the same launch code as an eager V-cycle (stream capture into the
// loop body) and rebuilt when the multigrid options change.
#include <math.h>
#include <stdlib.h>

#include <vector>

#include "qdeq_internal.cuh"

namespace qd {

// declared in mg.cu
__global__ void k_final_sum(const double *partial, int n, double *out);

struct SolveGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    qd_mg_options opt;
    bool net = false;   // built with the network's conditional correction
    double net_ratio = 0.0;
    int tail_sweeps = 0;
    double smooth_ratio = 0.0;
};

// n_kernels: kernels of the prologue, this one included; in_graph: set the
// loop condition (otherwise the host reads st->go)
// (phase: see solve_begin_dev; phase 1 also sets h_net)
__global__ void k_solve_begin(cudaGraphConditionalHandle h, cudaGraphConditionalHandle h_net, const double *scal,
                              SolveState *st, int rel, double tol, int n_kernels, int in_graph, int phase,
                              double net_ratio) {
    const int go = solve_begin_dev(sqrt(scal[0]), rel ? sqrt(scal[1]) : 0.0, st, rel, tol, n_kernels, phase, net_ratio);
    if (in_graph) {
        cudaGraphSetConditional(h, go ? 1u : 0u);
        if (phase == 1) cudaGraphSetConditional(h_net, st->net ? 1u : 0u);
    }
}

// n_kernels: kernels of one loop iteration, this one included
__global__ void k_solve_check(cudaGraphConditionalHandle h, const double *scal, SolveState *st,
                              int max_cycles, int n_kernels, int in_graph) {
    const int go = solve_check_dev(sqrt(scal[0]), st, max_cycles, n_kernels);
    if (in_graph) cudaGraphSetConditional(h, go ? 1u : 0u);
}

static bool same_opts(const qd_mg_options &a, const qd_mg_options &b) {
    return a.n_levels == b.n_levels && a.nu_pre == b.nu_pre && a.nu_post == b.nu_post &&
           a.nu_coarse == b.nu_coarse && a.tol_mode == b.tol_mode && a.tol == b.tol &&
           a.max_cycles == b.max_cycles && a.precision == b.precision &&
           a.surface_prolong == b.surface_prolong && a.coarse_solve == b.coarse_solve;
}

// The solver's instantiated solve graphs: [0] without the network's
// correction, [1] with it (a predicting solver switches between them when
// the warm start stands by, see warm_start_standby_update)
struct SolveGraphs {
    SolveGraph *g[2] = {nullptr, nullptr};
};

static void graph_free(SolveGraph *g) {
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
}

void solve_graph_free(qd_solver *s) {
    SolveGraphs *gs = static_cast<SolveGraphs *>(s->solve_graph);
    if (!gs) return;
    graph_free(gs->g[0]);
    graph_free(gs->g[1]);
    delete gs;
    s->solve_graph = nullptr;
}

// The cycle cap a solve's decision kernels apply.  The host-driven loop
// (eager mode) honours max_cycles <= 0 as "no cap", as the reference's loop
// (odeSolver.cpp:696) does; inside the solve graph the loop runs on the
// device with no host check, so there an uncapped solve stops after
// QD_SOLVE_GRAPH_MAX_CYCLES cycles and reports QD_ERR_NOT_CONVERGED.
static int cycle_cap(const qd_solver *s, int in_graph) {
    if (s->opt.max_cycles > 0) return s->opt.max_cycles;
    return in_graph ? QD_SOLVE_GRAPH_MAX_CYCLES : 0;
}

// the mixed solver's check after a correction: the level-0 residual ->
// FP32 rhs, its norm and the loop's decision in the residual's last block
// (and, with the smoothing pass enabled, whether the next correction is
// one: h_smooth); n_cycle / n_smooth: the kernels of a V-cycle iteration
// and of a smoothing iteration before the check
static int mixed_check(qd_solver *s, cudaGraphConditionalHandle h, cudaGraphConditionalHandle h_smooth,
                       int in_graph, int n_cycle, int n_smooth, const int *gate = nullptr) {
    Decide dc{};
    dc.gate = gate;
    dc.mode = 2;
    dc.max_cycles = cycle_cap(s, in_graph);
    dc.n_kernels = n_cycle + 1;
    dc.n_kernels_smooth = n_smooth + 1;
    dc.smooth_ratio = s->smooth_ratio;
    dc.in_graph = in_graph;
    dc.h = h;
    dc.h_smooth = h_smooth;
    dc.st = s->d_solve;
    return level0_norm_decide(s, dc);
}

// the body of one loop iteration: a V-cycle (or, smooth, the mixed
// solver's level-0 smoothing pass) and the norm of the new residual; in
// mixed precision the norm's last block also takes the loop's decision
// (*fused set), otherwise k_solve_check follows
static int capture_cycle(qd_solver *s, cudaGraphConditionalHandle h, int in_graph, long long launches0,
                         bool *fused, bool smooth = false) {
    *fused = false;
    if (s->opt.precision == QD_PREC_MIXED) {
        if (smooth)
            QD_TRY(smooth32_into64(s));      // level-0 sweeps on A e = r from zero, then u += e
        else
            QD_TRY(vcycle32_into64(s));      // FP32 cycle on A e = r, then u += e
        const int n = (int)(s->launches - launches0);
        QD_TRY(mixed_check(s, h, 0, in_graph, n, n));
        *fused = true;
    } else {
        int nb = 0;
        QD_TRY(vcycle64_norm(s, &nb));       // the last kernel leaves norm partials
        if (nb > 0) {
            k_final_sum<<<1, 1024, 0, s->stream>>>(s->d_partial, nb, s->d_scal);
            QD_LAUNCH_CHECK(s);
        } else {
            QD_TRY(level0_norm(s, 0, 0));
        }
    }
    return QD_OK;
}

// the solve's prologue: ||r0|| (relative tolerance), ||r|| of the guess and
// the first decision; in mixed precision one kernel (the residual's last
// block computes ||r0|| and decides), in FP64 k_r0, the norm and
// k_solve_begin.  n_kernels counts the prologue's kernels and `extra`
// kernels launched before it; phase as for solve_begin_dev.
static int prologue(qd_solver *s, cudaGraphConditionalHandle h, cudaGraphConditionalHandle h_net, int in_graph,
                    long long launches0, int extra, int phase, int n_gated = 0) {
    const int rel = s->opt.tol_mode == QD_TOL_REL;
    if (s->opt.precision == QD_PREC_MIXED) {
        Decide dc{};
        dc.mode = 1;
        dc.rel = rel;
        dc.tol = s->opt.tol;
        dc.n_kernels = (int)(s->launches - launches0) + 1 + extra;
        dc.n_kernels_gated = n_gated;
        dc.in_graph = in_graph;
        dc.phase = phase;
        dc.net_ratio = s->net_ratio;
        dc.h = h;
        dc.h_net = h_net;
        dc.st = s->d_solve;
        return level0_norm_decide(s, dc);
    }
    if (rel) QD_TRY(r0_norm(s, 1));
    QD_TRY(level0_norm(s, 0, 0));
    k_solve_begin<<<1, 1, 0, s->stream>>>(h, h_net, s->d_scal, s->d_solve, rel, s->opt.tol,
                                          (int)(s->launches - launches0) + 1 + extra, in_graph, phase,
                                          s->net_ratio);
    QD_LAUNCH_CHECK(s);
    return QD_OK;
}

// the network's correction of the guess and the prologue again (the body
// of the graph's IF node, or its eager form)
static int corrected_prologue(qd_solver *s, cudaGraphConditionalHandle h, int in_graph, long long launches0,
                              int n_gated = 0) {
    int nk = 0;
    QD_TRY(warm_start_predict(s, &nk));
    return prologue(s, h, 0, in_graph, launches0, nk, 2, n_gated);
}

static int end_capture(qd_solver *s, cudaGraph_t *g, int rc) {
    cudaGraph_t out = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s->stream, &out);
    if (rc != QD_OK) return rc;
    QD_CUDA(e);
    if (g) *g = out;
    return QD_OK;
}

// the node of a captured chain in g that nothing depends on
static int chain_leaf(cudaGraph_t g, cudaGraphNode_t *leaf) {
    size_t n = 0;
    QD_CUDA(cudaGraphGetNodes(g, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    QD_CUDA(cudaGraphGetNodes(g, nodes.data(), &n));
    *leaf = nullptr;
    for (auto nd : nodes) {
        size_t nout = 0;
        QD_CUDA(cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &nout));
        if (nout == 0) *leaf = nd;
    }
    return QD_OK;
}

// The kernels of one mixed-precision V-cycle (captured into a throwaway
// graph and counted).
static int count_cycle_kernels(qd_solver *s, int *n) {
    const long long l0 = s->launches;
    cudaGraph_t tmp = nullptr;
    QD_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeRelaxed));
    const int rc = vcycle32_into64(s);
    *n = (int)(s->launches - l0);
    s->launches = l0;
    QD_TRY(end_capture(s, &tmp, rc));
    if (tmp) cudaGraphDestroy(tmp);
    return QD_OK;
}

// One solve graph:
//   prologue -> [IF net: correction, prologue] -> loop
// In FP64 the loop is a WHILE node whose body is a V-cycle and the check.
// Each evaluation of a conditional node has a fixed cost (on GB300, around
// empty kernels: a WHILE node of one iteration about 10 us more than a plain
// kernel, an untaken IF node about 12 us), most of which a solve's own
// kernels hide, and with the history guess nearly every mixed-precision
// solve takes exactly one V-cycle.  So in mixed precision the first V-cycle
// and its check follow the prologue as plain nodes, their kernels skipping
// themselves when the prologue found the guess converged (they read
// SolveState.go), and only the corrections after the first run in the
// WHILE node -- each a V-cycle, or with the smoothing pass enabled an
// IF/ELSE node choosing the pass or a V-cycle, then the check.  (Measured
// on the rupture window at 1025^2: about 1 % of a step.)
static int build(qd_solver *s, SolveGraph *sg) {
    QD_CUDA(cudaGraphCreate(&sg->graph, 0));
    cudaGraphConditionalHandle h, h_net = 0, h_smooth = 0;
    QD_CUDA(cudaGraphConditionalHandleCreate(&h, sg->graph, 0, cudaGraphCondAssignDefault));
    sg->net = warm_start_predicting(s);
    sg->net_ratio = s->net_ratio;
    if (sg->net) QD_CUDA(cudaGraphConditionalHandleCreate(&h_net, sg->graph, 0, cudaGraphCondAssignDefault));
    const bool mixed = s->opt.precision == QD_PREC_MIXED;
    const bool smooth = mixed && s->smooth_ratio > 1.0;
    if (smooth) QD_CUDA(cudaGraphConditionalHandleCreate(&h_smooth, sg->graph, 0, cudaGraphCondAssignDefault));
    int n_cycle = 0;
    if (mixed) QD_TRY(count_cycle_kernels(s, &n_cycle));
    const int n_gated = mixed ? n_cycle + 1 : 0;
    // prologue, captured into the top-level graph
    // captured launches are counted on the device each time they run, so the
    // host counter is restored after each capture
    const long long launches0 = s->launches;
    QD_CUDA(cudaStreamBeginCaptureToGraph(s->stream, sg->graph, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeRelaxed));
    int rc = prologue(s, h, h_net, 1, launches0, 0, sg->net ? 1 : 0, n_gated);
    s->launches = launches0;
    QD_TRY(end_capture(s, nullptr, rc));
    // the prologue is a chain: its one leaf is the next node's dependency
    cudaGraphNode_t leaf = nullptr;
    QD_TRY(chain_leaf(sg->graph, &leaf));
    if (sg->net) {
        // IF the guess misses the tolerance by more than the gate: the
        // network's correction and the prologue on the corrected guess
        // (which re-sets the loop's condition)
        cudaGraphNodeParams ip = {};
        ip.type = cudaGraphNodeTypeConditional;
        ip.conditional.handle = h_net;
        ip.conditional.type = cudaGraphCondTypeIf;
        ip.conditional.size = 1;
        cudaGraphNode_t gate;
        QD_CUDA(cudaGraphAddNode(&gate, sg->graph, leaf ? &leaf : nullptr, nullptr, leaf ? 1 : 0, &ip));
        QD_CUDA(cudaStreamBeginCaptureToGraph(s->stream, ip.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeRelaxed));
        rc = corrected_prologue(s, h, 1, launches0, n_gated);
        s->launches = launches0;
        QD_TRY(end_capture(s, nullptr, rc));
        leaf = gate;
    }
    if (mixed) {
        // the first V-cycle and its check, skipped by their kernels when
        // the prologue found the guess converged (SolveState.go = 0, and
        // the prologue then set the loop's condition to 0)
        QD_CUDA(cudaStreamBeginCaptureToGraph(s->stream, sg->graph, leaf ? &leaf : nullptr, nullptr, leaf ? 1 : 0,
                                              cudaStreamCaptureModeRelaxed));
        s->cycle_gate = &s->d_solve->go;
        rc = vcycle32_into64(s);
        if (rc == QD_OK) rc = mixed_check(s, h, h_smooth, 1, n_cycle, 1, &s->d_solve->go);
        s->cycle_gate = nullptr;
        s->launches = launches0;
        QD_TRY(end_capture(s, nullptr, rc));
        cudaGraphNode_t last = nullptr;
        QD_TRY(chain_leaf(sg->graph, &last));
        leaf = last;
    }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t loop;
    QD_CUDA(cudaGraphAddNode(&loop, sg->graph, leaf ? &leaf : nullptr, nullptr, leaf ? 1 : 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if (smooth) {
        // body: IF the check chose the smoothing pass THEN that pass ELSE a
        // V-cycle; then the check (residual, norm, both decisions)
        cudaGraphNodeParams ep = {};
        ep.type = cudaGraphNodeTypeConditional;
        ep.conditional.handle = h_smooth;
        ep.conditional.type = cudaGraphCondTypeIf;
        ep.conditional.size = 2;
        cudaGraphNode_t branch;
        QD_CUDA(cudaGraphAddNode(&branch, body, nullptr, nullptr, 0, &ep));
        QD_CUDA(cudaStreamBeginCaptureToGraph(s->stream, ep.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeRelaxed));
        rc = smooth32_into64(s);
        const int n_smooth = (int)(s->launches - launches0);
        s->launches = launches0;
        QD_TRY(end_capture(s, nullptr, rc));
        QD_CUDA(cudaStreamBeginCaptureToGraph(s->stream, ep.conditional.phGraph_out[1], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeRelaxed));
        rc = vcycle32_into64(s);
        s->launches = launches0;
        QD_TRY(end_capture(s, nullptr, rc));
        QD_CUDA(cudaStreamBeginCaptureToGraph(s->stream, body, &branch, nullptr, 1, cudaStreamCaptureModeRelaxed));
        rc = mixed_check(s, h, h_smooth, 1, n_cycle, n_smooth);
        s->launches = launches0;
        QD_TRY(end_capture(s, nullptr, rc));
    } else {
        QD_CUDA(cudaStreamBeginCaptureToGraph(s->stream, body, nullptr, nullptr, 0,
                                              cudaStreamCaptureModeRelaxed));
        bool fused = false;
        rc = capture_cycle(s, h, 1, launches0, &fused);
        if (rc == QD_OK && !fused) {
            const int n = (int)(s->launches - launches0) + 1;
            k_solve_check<<<1, 1, 0, s->stream>>>(h, s->d_scal, s->d_solve, cycle_cap(s, 1), n, 1);
            if (cudaPeekAtLastError() != cudaSuccess) rc = QD_ERR_CUDA;
        }
        s->launches = launches0;
        QD_TRY(end_capture(s, nullptr, rc));
    }
    QD_CUDA(cudaGraphInstantiate(&sg->exec, sg->graph, 0));
    sg->opt = s->opt;
    sg->tail_sweeps = s->tail_sweeps;
    sg->smooth_ratio = s->smooth_ratio;
    return QD_OK;
}

// The same solve with the loop on the host: every kernel is an ordinary
// stream launch and the host reads the decision after each cycle.  Chosen
// by QDEQ_EAGER_SOLVE=1, for per-kernel profilers that do not descend into
// conditional graph nodes; the kernels and their order are the graph's.
static bool eager_solve() {
    static const bool on = [] {
        const char *e = getenv("QDEQ_EAGER_SOLVE");
        return e && e[0] == '1';
    }();
    return on;
}

static int solve_eager(qd_solver *s) {
    const long long launches0 = s->launches;
    const bool net = warm_start_predicting(s);
    QD_TRY(prologue(s, 0, 0, 0, launches0, 0, net ? 1 : 0));
    s->launches = launches0;       // counted on the device, as in the graph
    if (net) {
        SolveState st;
        QD_TRY(solve_state_read(s, &st));
        if (st.net) {
            QD_TRY(corrected_prologue(s, 0, 0, launches0));
            s->launches = launches0;
        }
    }
    for (;;) {
        SolveState st;
        QD_TRY(solve_state_read(s, &st));
        if (!st.go) return QD_OK;
        bool fused = false;
        QD_TRY(capture_cycle(s, 0, 0, launches0, &fused, st.smooth != 0));
        if (!fused) {
            k_solve_check<<<1, 1, 0, s->stream>>>(0, s->d_scal, s->d_solve, cycle_cap(s, 0),
                                                  (int)(s->launches - launches0) + 1, 0);
            QD_LAUNCH_CHECK(s);
        }
        s->launches = launches0;
    }
}

// Enqueue one solve on the solver's stream (no host synchronisation).
int mg_solve_async(qd_solver *s) {
    if (warm_start_predicting(s)) s->net_armed_solves++;
    if (eager_solve()) return solve_eager(s);
    SolveGraphs *gs = static_cast<SolveGraphs *>(s->solve_graph);
    if (!gs) {
        gs = new SolveGraphs();
        s->solve_graph = gs;
    }
    const int key = warm_start_predicting(s) ? 1 : 0;
    SolveGraph *&sg = gs->g[key];
    if (sg && (!same_opts(sg->opt, s->opt) || sg->net_ratio != s->net_ratio || sg->tail_sweeps != s->tail_sweeps ||
               sg->smooth_ratio != s->smooth_ratio)) {
        graph_free(sg);
        sg = nullptr;
    }
    if (!sg) {
        sg = new SolveGraph();
        const int rc = build(s, sg);
        if (rc != QD_OK) {
            graph_free(sg);
            sg = nullptr;
            return rc;
        }
    }
    QD_CUDA(cudaGraphLaunch(sg->exec, s->stream));
    return QD_OK;
}

// Fetch the solve state (synchronises the stream).
int solve_state_read(qd_solver *s, SolveState *out) {
    QD_CUDA(cudaMemcpyAsync(s->h_solve, s->d_solve, sizeof(SolveState), cudaMemcpyDeviceToHost,
                            s->stream));
    QD_CUDA(cudaStreamSynchronize(s->stream));
    *out = *s->h_solve;
    return QD_OK;
}

int solve_state_clear_flag(qd_solver *s) {
    QD_CUDA(cudaMemsetAsync(&s->d_solve->flag, 0, sizeof(int), s->stream));
    return QD_OK;
}

// multigrid(): one solve, then its outcome
int mg_solve(qd_solver *s, int *cycles, double *rnorm, double *r0norm) {
    QD_TRY(solve_state_clear_flag(s));
    QD_TRY(mg_solve_async(s));
    SolveState st;
    QD_TRY(solve_state_read(s, &st));
    if (cycles) *cycles = st.cycles;
    if (rnorm) *rnorm = st.delta;
    if (r0norm) *r0norm = st.r0;
    if (st.flag & 1) {
        set_error("multigrid: residual norm is %f after %d cycles", st.delta, st.cycles);
        return QD_ERR_NOT_CONVERGED;
    }
    if (st.flag & 2) {
        set_error("multigrid: %d cycles, ||r|| = %.3e > %.3e", st.cycles, st.delta, st.thr);
        return QD_ERR_NOT_CONVERGED;
    }
    return QD_OK;
}

}  // namespace qd
