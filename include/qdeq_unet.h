/* qdeq_unet.h -- the learned warm start of the GB300 hot path.
 *
 * A 4-level U-Net (16/32/64/128 channels, 3x3 convolutions, BF16 weights and
 * activations, FP32 accumulation on the 5th-generation tensor cores) that
 * predicts the change a stage's multigrid solve will make to the
 * displacement field u, from the field the solve starts at and the stage's
 * change of the Dirichlet data on the fault and far columns.  The multigrid
 * always iterates from the predicted field to the same residual tolerance,
 * so the prediction only changes the V-cycle count, never the result's
 * tolerance.  The reference has no counterpart to anything in this header.
 *
 * Parameters are flat FP32 arrays: for each of the 15 convolutions in order
 * (encoder 8, decoder 6, head 1), weights [9 taps][cout][cin] (tap = 3*(dy+1)
 * + (dx+1)) followed by the bias [cout].  The first layer has cin = 16 (five
 * input channels used), the head cout = 16 (channel 0 used).
 * Host inputs are planar float arrays over the nk x ni level-0 grid:
 * x = [5][nk][ni] input channels, target / y = [nk][ni].  Attached to a
 * solver the inputs are u / (largest boundary value), the change of the
 * fault and far Dirichlet data (each over s, the largest such change)
 * broadcast along the rows, the column position, and the change the
 * previous solve made to u over that solve's s; the target is the change
 * this solve makes to u, over s.
 */
#ifndef QDEQ_UNET_H
#define QDEQ_UNET_H

#include "qdeq.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qd_unet qd_unet;

/* A network for an nk x ni grid ((nk-1) and (ni-1) divisible by 8), with
 * seeded He-normal weights (the head and the unused input channels start at
 * zero, so a fresh network predicts no change). */
int qd_unet_create(int nk, int ni, unsigned long long seed, qd_unet **out);
void qd_unet_destroy(qd_unet *u);
long long qd_unet_num_params(const qd_unet *u);
int qd_unet_get_params(qd_unet *u, float *host);
int qd_unet_set_params(qd_unet *u, const float *host);

/* y = network(x), on the host arrays (device round trip) */
int qd_unet_forward_host(qd_unet *u, const float *x, float *y);

/* loss = mean over the grid of (y - target)^2 and its gradient with respect
 * to every parameter (grads: num_params floats, may be NULL) */
int qd_unet_loss_grad_host(qd_unet *u, const float *x, const float *target, float *loss, float *grads);

/* one Adam step (beta 0.9 / 0.999) with learning rate lr on (x, target) */
int qd_unet_train_step_host(qd_unet *u, const float *x, const float *target, float lr, float *loss);

/* Attach the network to a solver of the same grid, or of twice or four
 * times its resolution (2n-1 or 4n-3 nodes per side for an n-node network:
 * the network then sees every other or every fourth level-0 node -- the
 * multigrid's level-1 or level-2 grid -- and its prediction is interpolated
 * bilinearly; each halving of the resolution cuts the cost about four
 * times).  Mode 1 trains
 * online (one Adam step per stage solve on the change the solve made, the
 * solve itself starting from the unmodified field), mode 2 predicts, mode 0
 * detaches.  In mode 2 each stage solve first measures the residual of its
 * guess; when that misses the solve's threshold by more than the gate
 * (qd_solver_warm_start_gate) the solve adds the network's prediction,
 * scaled by the step that minimises the energy norm of the guess's error
 * (so the corrected guess is never worse in that norm), and iterates from
 * there; otherwise the network is left out.  The decision is taken on the
 * device, inside the solve's CUDA graph.  While attached the network runs
 * on the solver's stream; destroying the solver detaches it. */
int qd_solver_warm_start(qd_solver *s, qd_unet *u, int mode, float lr);

/* The gate of mode 2: the network corrects a solve's guess only when the
 * guess's residual norm exceeds ratio x the solve's threshold (ratio >= 1).
 * ratio 0 (the default): the measured rule -- when the guess would need more
 * than 1 + c V-cycles to reach the threshold, c the network's cost in
 * V-cycles (qd_solver_warm_start_cost, default 2); the ratio is then
 * rho^-(1 + c), rho the solver's running geometric mean of the residual
 * reduction per V-cycle (measured on the device; 1 until a cycle has run).
 * A correction can only pay where the cycles it saves cost more than the
 * inference.  qd_stats.net_cycles_needed / net_cycles_taken report, over the
 * corrected solves, the cycles their guesses needed and those they took.
 * Under the measured rule the RK43 driver also stands the network by for
 * the next attempt when no solve of an attempt had a guess that needed it:
 * those solves run the solve graph without the network's conditional node
 * (it would have been left out of all of them), and the first guess that
 * needs it brings the network's graph back for the attempt after. */
int qd_solver_warm_start_gate(qd_solver *s, double ratio);
/* The measured rule's cost of one correction in V-cycles (>= 0; 0 gives
 * the rule "when one V-cycle would not reach the threshold"); selects the
 * measured rule. */
int qd_solver_warm_start_cost(qd_solver *s, double cycles);

/* training steps taken, and the loss of the last step */
int qd_unet_stats(qd_unet *u, long long *train_steps, float *last_loss);

/* Mean device microseconds of one inference (what = 0), one training step
 * without the parameter update (what = 1: forward, loss, backward) or the
 * first convolution alone (what = 2: 16 -> 16 channels on the full grid,
 * the network's most frequent and longest-running kernel), timed with CUDA
 * events over `reps` back-to-back runs on the network's stream on its
 * current input and target; *flops receives the tensor-core FLOPs of one
 * run (2 * 9 * cin * cout per output pixel of every convolution; in
 * training, the data and weight gradients add two more). */
int qd_unet_time(qd_unet *u, int what, int reps, double *us, double *flops);

#ifdef __cplusplus
}
#endif

#endif
