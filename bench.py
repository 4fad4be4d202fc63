#!/usr/bin/env python
"""Benchmark: simulated years per wall-hour of the quasi-dynamic earthquake
cycle at 1025 x 1025 (config 1 physics: layered mu, +-5% a-b perturbation,
8-level multigrid, 1e-9 relative residual).

A "step" is one accepted adaptive-RK43 step: the ARK4(3)6L stages, each an
elliptic multigrid solve plus the fault stress / Newton / aging-law update,
retried until the error test passes, then the refresh solve at the new state.
Every GPU run starts from the steady-sliding initial state (V = Vp), takes W
untimed warm-up steps and times the next K steps.  The learned warm start's
U-Net is first trained online for T accepted steps (--train-steps) on a
separate instance of the workload (another seed of the a-b perturbation),
one Adam step per stage solve; the timed run then starts every stage solve
from the network's prediction.  value = simulated years advanced in the timed steps / their device
time in hours.

Arms:
  default           this library on the GPU: the learned warm start with FP32
                    V-cycles in FP64 refinement (the headline); the same
                    solver without the network, and the plain FP64 multigrid,
                    are measured on the same steps
  --impl reference  the reference algorithm on the host cores (the CPU
                    oracle restating odeSolver.cpp / fault.cpp: 6 levels,
                    V(32,32)), same config, same steps

The L2 cache (129 MB, larger than the 1025^2 working set) is flushed before
every timed step by writing a 512 MB buffer outside the timed interval.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

YEAR_S = 365.25 * 86400.0
# DRAM bytes (read + write) per launch from ncu captures with the caches
# flushed before the kernel: the V-cycle kernels of the mixed solver at
# 1025^2 (profiles/vcycle_kernels_1025.md) and the U-Net's first 16 -> 16
# channel convolution on the network's grid (profiles/unet_conv_1025.md),
# keyed by the network's nodes per side
TRAFFIC = {"up0": 31.19e6, "down0": 17.35e6, "residual": 33.74e6}
TRAFFIC_CONV16 = {513: 8.62e6, 1025: 34.03e6}
METRIC = "simulated yr/hr at 1025² (learned+mixed vs plain FP64 MG, 1e-9 rel residual)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", default="config1")
    p.add_argument("--cpu-sample-s", type=float, default=20.0)
    p.add_argument("--ref-budget-s", type=float, default=60.0,
                   help="--impl reference: stop timing after the step that passes this many seconds")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--headline-only", action="store_true",
                   help="time only the headline solver (no FP64 comparison, e2e or CPU runs)")
    p.add_argument("--train-steps", type=int, default=100,
                   help="accepted steps of online training on a separate instance of the workload")
    p.add_argument("--no-learned", action="store_true", help="headline without the learned warm start")
    p.add_argument("--lr", type=float, default=1e-3)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--profile-run", action="store_true",
                   help="only the headline solver's W + K steps (network trained for --train-steps "
                        "steps first), for per-kernel profilers; prints a one-line summary")
    p.add_argument("--autotune", action="store_true",
                   help="qd_autotune the single-instance runs with the history guess after their warm-up "
                        "(by default they keep the config's V(2,2) and the default tiles, which time faster "
                        "on this workload than the tuner's picks; the ensemble is always tuned per instance)")
    p.add_argument("--no-autotune", action="store_true",
                   help="no tuning anywhere, the ensemble's instances included")
    p.add_argument("--schedule", default=None,
                   help="nu_pre,nu_post of the fast runs (no tuning of them)")
    p.add_argument("--net-gate", type=float, default=0.0,
                   help="the network corrects a stage solve's guess when the guess's residual exceeds "
                        "this multiple of the solve's threshold (0: when one V-cycle at the solver's "
                        "measured reduction per cycle would not reach it)")
    p.add_argument("--unet-level", type=int, default=1, choices=[0, 1, 2],
                   help="multigrid level whose grid the U-Net runs on (1: every other node, its "
                        "prediction prolongated bilinearly)")
    p.add_argument("--history", type=int, default=4,
                   help="stored solutions of the solution-history guess (0: start every solve "
                        "from the previous solution, as the reference)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU arm: the reference algorithm through the oracle
# ---------------------------------------------------------------------------
def reference_mg_for(cfg):
    from qdeqcycle_fdm_gb300 import config
    r = config.reference_mg()
    r.tol_mode, r.tol = cfg.mg.tol_mode, cfg.mg.tol      # same accuracy target as the GPU arm
    r.max_cycles = 0
    return r


def run_cpu(prob, warmup, steps, budget_s=None):
    """Oracle RK43 from t = 0: `warmup` untimed steps, then up to `steps`
    timed steps (stopping early once budget_s of timed work is spent)."""
    import oracle
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    mg = reference_mg_for(prob.cfg)
    sim = oracle.Simulation(prob, mg.n_levels, mg.nu_pre, mg.nu_post, mg.nu_coarse, mg.tol_mode,
                            mg.tol, mg.max_cycles)
    sim.start()
    for _ in range(warmup):
        sim.step()
    s0 = sim.state()
    t0 = time.perf_counter()
    n = 0
    while n < steps:
        sim.step()
        n += 1
        if budget_s is not None and time.perf_counter() - t0 > budget_s:
            break
    wall = time.perf_counter() - t0
    s1 = sim.state()
    yrs = (s1["t"] - s0["t"]) / YEAR_S
    return {"value": yrs / (wall / 3600.0) if wall > 0 else 0.0, "wall_s": wall, "steps": n,
            "sim_years": yrs, "threads": threads,
            "vcycles_per_solve": (s1["vcycles"] - s0["vcycles"]) / max(1, s1["solves"] - s0["solves"]),
            "schedule": f"{mg.n_levels} levels V({mg.nu_pre},{mg.nu_post}), rel {mg.tol:g}"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from qdeqcycle_fdm_gb300 import config, problem
    import oracle
    oracle.build(ref=False)
    cfg = config.CONFIGS[args.config]()
    prob = problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])
    r = run_cpu(prob, args.warmup, args.steps, budget_s=args.ref_budget_s)
    line = {
        "impl": "reference", "metric": METRIC, "value": r["value"], "unit": "sim_yr/hr",
        "n_gpus": args.gpus, "steps": r["steps"], "warmup": args.warmup,
        "ms_per_step": 1e3 * r["wall_s"] / max(1, r["steps"]), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{cfg.name}: {cfg.ni}x{cfg.nk} earthquake cycle, accepted RK43 steps "
                               f"{args.warmup + 1}..{args.warmup + r['steps']} from steady sliding",
                   "mg": r["schedule"], "l2": "host run"},
        "cpu_baseline": {"value": r["value"], "unit": "sim_yr/hr", "cores": r["threads"],
                         "kind": "port",
                         "sample": f"{r['steps']} accepted steps after {args.warmup} warm-up steps"},
        "e2e": {"value": r["value"], "unit": "sim_yr/hr", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "vcycles_per_solve": r["vcycles_per_solve"],
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch

    from qdeqcycle_fdm_gb300 import api, build, config, problem, replicas, warmstart
    rank, world, local = replicas.env()
    torch.cuda.set_device(local)
    replicas.init("nccl")          # replicas only: the data path has no collective
    build.build()
    cfg = config.CONFIGS[args.config]()
    prob = problem.build_problem(cfg)            # face moduli homogenised on the GPU
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    T = args.train_steps
    H = args.history

    def unet_n(n):
        """network nodes per side: the solver's level-0 grid, or its level-1
        grid with the prediction prolongated bilinearly"""
        return (n - 1) // (1 << args.unet_level) + 1
    TUNE = args.autotune and not args.no_autotune and args.schedule is None
    TUNE_ENSEMBLE = not args.no_autotune

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def train_network(mg):
        """Online training on a separate instance of the workload (the same
        physics with another seed of the a-b perturbation): T accepted steps
        from steady sliding, one Adam step per stage solve.  The timed runs
        then use the network on the benchmark instance, whose states it has
        not seen."""
        tcfg = cfg.replace(seed=cfg.seed + 1)
        tprob = problem.build_problem(tcfg)
        tsim = api.Simulation(tprob, mg)
        tsim.solver.set_solution_history(H)
        net = warmstart.UNet(unet_n(tprob.nk), unet_n(tprob.ni), seed=args.seed)
        net.attach(tsim.solver, warmstart.MODE_TRAIN, args.lr)
        tsim.start()
        tsim.step(T)
        n, loss = net.stats()
        net.attach(tsim.solver, warmstart.MODE_OFF)
        tsim.close()
        return net, {"train_samples": n, "last_loss": loss, "train_instance_seed": tcfg.seed}

    def timed_run(mg, host_io=False, net=None, history=0, tune=False):
        """W untimed warm-up steps from steady sliding, then K steps each
        bracketed by CUDA events on the solver's stream (L2 flushed before
        each); with `history` >= 2 every stage solve starts from the
        solution-history guess, and with `net` from the network's correction
        of that guess; `tune`: qd_autotune on the run's own state after the
        warm-up steps (outside the timed region).  host_io: every step goes
        through the C ABI with host
        buffers -- state and u uploaded from pinned memory before, read back
        after (the e2e measurement)."""
        sim = api.Simulation(prob, mg)
        sim.solver.set_solution_history(history)
        if net is not None:
            net.attach(sim.solver, warmstart.MODE_PREDICT)
            warmstart.UNet.set_gate(sim.solver, args.net_gate)
        sim.start()
        sim.step(args.warmup)
        tuning = sim.solver.autotune(3) if tune else None
        stream = torch.cuda.ExternalStream(sim.solver.stream_ptr())
        s0 = sim.state(with_u=False)
        ms, step_ms = 0.0, []
        if host_io:
            nz, nx = prob.nz, prob.nx

            def pinned(shape):
                return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

            hU = pinned((nz, nx))
            sim.solver.download_u(out=hU)
            hv = {k: pinned(nz) for k in ("Slip", "psi", "V", "dpsi", "Ts")}
            st = sim.solver.rk43_state(out=hv)
        barrier()
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if host_io:
                sim.solver.rk43_set_state(hv["Slip"], hv["psi"], hv["V"], hv["dpsi"], st["t"], st["dt"],
                                          st["errA"][0], st["errA"][1], st["it"])
                sim.solver.upload_u(hU)
                sim.solver.rk43_step(1)
                st = sim.solver.rk43_state(out=hv)
                sim.solver.download_u(out=hU)
            else:
                sim.step(1)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            ms += step_ms[-1]
        barrier()
        s1 = sim.state(with_u=False)
        if net is not None:
            net.attach(sim.solver, warmstart.MODE_OFF)
        return sim, {"ms": ms, "yrs": (s1["t"] - s0["t"]) / YEAR_S, "step_ms": step_ms,
                     "t0": s0["t"], "t_end": s1["t"],
                     "launches": s1["kernel_launches"] - s0["kernel_launches"],
                     "vcycles": s1["vcycles"] - s0["vcycles"], "solves": s1["solves"] - s0["solves"],
                     "net_solves": s1["net_solves"] - s0["net_solves"],
                     "attempts": s1["attempts"] - s0["attempts"], "autotune": tuning}

    def job_value(run):
        """whole-job simulated yr/hr: years of all replicas / slowest rank's hours"""
        return replicas.aggregate(run["yrs"], run["ms"] / 3.6e6, device="cuda")[2]

    def reduce_max(x):
        return replicas.aggregate(0.0, x, device="cuda")[1]

    def summary(run):
        return {"value": job_value(run), "ms_per_step": reduce_max(run["ms"]) / args.steps,
                "vcycles_per_solve": run["vcycles"] / max(1, run["solves"]),
                "sim_years_timed": run["yrs"]}

    mixed_cfg = config.MGConfig(**{**cfg.mg.__dict__, "precision": 1, "surface_prolong": 1,
                                   "coarse_solve": 1})
    if args.schedule:
        nu = [int(v) for v in args.schedule.split(",")]
        mixed_cfg = config.MGConfig(**{**mixed_cfg.__dict__, "nu_pre": nu[0], "nu_post": nu[1]})
    fp64_cfg = config.MGConfig(**{**cfg.mg.__dict__, "precision": 0, "surface_prolong": 0})
    fp64s_cfg = config.MGConfig(**{**cfg.mg.__dict__, "precision": 0, "surface_prolong": 1,
                                   "coarse_solve": 1})
    learned = not args.no_learned
    peaks = _peaks()
    net, tinfo = train_network(mixed_cfg) if learned else (None, {})
    if args.profile_run:
        simp, run = timed_run(mixed_cfg, net=net, history=H, tune=TUNE)
        simp.close()
        if rank == 0:
            print(json.dumps({"profile_run": "headline solver", "learned": learned, "history": H,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": run["ms"] / args.steps,
                              "vcycles_per_solve": run["vcycles"] / max(1, run["solves"]),
                              "solves_per_step": run["solves"] / args.steps,
                              "network_corrected_solves": run["net_solves"] / max(1, run["solves"]),
                              "autotune": run["autotune"]}),
                  flush=True)
        if net is not None:
            net.close()
        return 0
    clocks = Clocks(local)
    clocks.start()
    sim, head = timed_run(mixed_cfg, net=net, history=H, tune=TUNE)
    clk = clocks.stop()
    ms_max = reduce_max(head["ms"])
    value = job_value(head)
    extra = {}
    if learned:
        simm, mixed = timed_run(mixed_cfg, history=H, tune=TUNE)
        simm.close()
        extra["mixed_no_learned"] = summary(mixed)
        us_f, fl_f = net.time("forward", 10)
        us_t, fl_t = net.time("train", 5)
        bf = peaks.get("bf16_tflops", 1900.0)
        extra["warm_start"] = {
            "network": "U-Net 4 levels 16/32/64/128 ch, 3x3 conv, BF16 in / FP32 accumulate (tcgen05)",
            "network_grid": f"{unet_n(prob.nk)}x{unet_n(prob.ni)} (multigrid level {args.unet_level}"
                            + (", prediction prolongated bilinearly)" if args.unet_level else ")"),
            "train_steps": T, **tinfo, "lr": args.lr,
            "inference_us": us_f, "inference_tflops": fl_f / (us_f * 1e-6) / 1e12,
            "train_step_us": us_t, "train_tflops": fl_t / (us_t * 1e-6) / 1e12,
            "tensor_peak_tflops": bf, "inference_frac_of_peak": fl_f / (us_f * 1e-6) / 1e12 / bf}
    if H >= 2 and not args.headline_only:
        simp, prev = timed_run(mixed_cfg)
        simp.close()
        extra["mixed_previous_solution_start"] = summary(prev)
    if args.headline_only:
        args.no_e2e = args.no_cpu_baseline = True
        plain = plain_s = None
        plain_value = None
    else:
        sim64, plain = timed_run(fp64_cfg)
        sim64.close()
        sim64s, plain_s = timed_run(fp64s_cfg)
        sim64s.close()
        plain_value = plain["yrs"] / (reduce_max(plain["ms"]) / 3.6e6)

    def ensemble_run(ksteps=8):
        """Config 4 in miniature: 12 x 257^2 + 6 x 513^2 + 2 x 1025^2 seeded
        instances (each its own parameters and adaptive dt), advanced by
        qd_ensemble_step (GPU work of all instances interleaved) and, for
        comparison, one instance after the other.  Host wall clock with the
        device synchronised on both sides (the instances use 20 streams)."""
        sizes = [257] * 12 + [513] * 6 + [1025] * 2
        cfgs = [config.ensemble_instance(n, i) for i, n in enumerate(sizes)]
        probs = [problem.build_problem(c) for c in cfgs]
        out = {"instances": "12 x 257^2 + 6 x 513^2 + 2 x 1025^2 (config-4 parameter draws)",
               "steps_timed": ksteps, "warmup": 3, "history": H,
               "autotune": "per instance" if TUNE_ENSEMBLE else None}
        for mode in ("batched", "sequential"):
            sims = [api.Simulation(p, c.mg) for p, c in zip(probs, cfgs)]
            for x in sims:
                x.solver.set_solution_history(H)
                x.start()
            if mode == "batched":
                api.ensemble_step(sims, 3)
            else:
                for x in sims:
                    x.step(3)
            if TUNE_ENSEMBLE:
                for x in sims:
                    x.solver.autotune(2)          # on each instance's own state, untimed
            t0 = [x.solver.rk43_state()["t"] for x in sims]
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            if mode == "batched":
                api.ensemble_step(sims, ksteps)
            else:
                for x in sims:
                    x.step(ksteps)
            torch.cuda.synchronize()
            wall = time.perf_counter() - w0
            yrs = sum(x.solver.rk43_state()["t"] - a for x, a in zip(sims, t0)) / YEAR_S
            out[mode] = {"wall_s": wall, "ms_per_ensemble_step": 1e3 * wall / ksteps,
                         "instance_years_per_hr": yrs / (wall / 3600.0)}
            for x in sims:
                x.close()
        out["batched_speedup"] = out["sequential"]["wall_s"] / out["batched"]["wall_s"]
        return out

    if not args.headline_only:
        extra["ensemble"] = ensemble_run()

    # Roofline.  The candidates are the kernels with the largest device time
    # in the headline step: the V-cycle's level-0 kernels and coarse tail and,
    # with the network, its first (full-grid, 16 -> 16 channel) convolution,
    # four of which run per inference.  Inside a solve the V-cycle kernels run
    # in a CUDA graph, so each is timed by qd_mg_time_kernel: REPS
    # back-to-back launches on the solver's stream between two CUDA events,
    # on the solver's own state after the timed run; the convolution by
    # qd_unet_time the same way.  Algorithmic bytes per launch are the
    # unfused algorithm's traffic:
    #   down0    nu_pre red+black sweeps x 20 B + residual/restriction 16 B
    #            per level-0 node, + 4 B per level-1 node
    #   up0      prolongation 8 B + nu_post sweeps x 20 B + u64 += e 16 B per
    #            level-0 node, + 4 B per level-1 node
    #            (nu_pre, nu_post: the schedule the run used, tuned or not)
    #   residual FP64 u, cx, cz, diag read + FP32 rhs written: 36 B per node
    #   conv16   16 BF16 channels read and written: 64 B per padded pixel of
    #            the network's grid
    # Launches per step: one of each cycle kernel per V-cycle, the residual
    # once more per solve (the guess) and once more per solve the network
    # corrected, the convolution 4 per corrected solve.  The dominant kernel
    # (largest time x launches per step) is the roofline entry.
    peak = peaks.get("hbm_gbs", 6800.0)
    n0 = cfg.ni * cfg.nk
    n1 = ((cfg.ni - 1) // 2 + 1) * ((cfg.nk - 1) // 2 + 1)
    # the network's padded grid (H+2 rows x W+2 columns rounded up to 8)
    pad_px = (unet_n(cfg.nk) + 2) * ((unet_n(cfg.ni) + 2 + 7) // 8 * 8)
    tn = head["autotune"]
    nu_pre, nu_post = (tn["nu_pre"], tn["nu_post"]) if tn else (mixed_cfg.nu_pre, mixed_cfg.nu_post)
    algo = {"up0": (24.0 + 20.0 * nu_post) * n0 + 4.0 * n1, "down0": (16.0 + 20.0 * nu_pre) * n0 + 4.0 * n1,
            "residual": 36.0 * n0,
            "conv16": 64.0 * pad_px}
    names = {"up0": f"k_up<float,2> level 0 (prolongation + {nu_post} sweep(s) + u64 += e)",
             "down0": f"k_down<float> level 0 ({nu_pre} sweep(s) + residual + restriction)",
             "residual": "k_residual64_to32 (FP64 residual -> FP32 rhs + norm)",
             "tail": "k_tail<float> (levels <= 65 rows, one CTA)",
             "conv16": f"k_conv_rows<16,16> (U-Net 3x3 convolution, {unet_n(cfg.nk)}x{unet_n(cfg.ni)} grid, tcgen05)"}
    REPS = 50
    kern = {}
    for k in ("up0", "down0", "residual", "tail"):
        sim.solver.time_kernel(k, 3)                      # warm-up launches
        kern[k] = {"us": sim.solver.time_kernel(k, REPS), "kernel": names[k]}
    cyc_step = head["vcycles"] / args.steps
    sol_step = head["solves"] / args.steps
    net_step = head["net_solves"] / args.steps
    per_step = {"up0": cyc_step, "down0": cyc_step, "residual": cyc_step + sol_step + net_step,
                "tail": cyc_step}
    if net is not None:
        net.time("conv16", 3)
        us_c, fl_c = net.time("conv16", REPS)
        kern["conv16"] = {"us": us_c, "kernel": names["conv16"],
                          "tflops": fl_c / (us_c * 1e-6) / 1e12}
        per_step["conv16"] = 4.0 * net_step
    for k, v in kern.items():
        v["launches_per_step"] = per_step[k]
        v["us_per_step"] = v["us"] * per_step[k]
        v["share_of_step_est"] = v["us_per_step"] / (1e3 * ms_max / args.steps)
        if k in algo:
            v["algo_bytes"] = algo[k]
            v["achieved_gbs"] = algo[k] / (v["us"] * 1e-6) / 1e9
    dom = max(algo.keys() & kern.keys(), key=lambda k: kern[k]["us_per_step"])
    achieved = kern[dom]["achieved_gbs"]
    traffic = TRAFFIC_CONV16.get(unet_n(cfg.nk)) if dom == "conv16" else TRAFFIC.get(dom)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "kernel": names[dom], "us_per_launch": kern[dom]["us"], "reps": REPS,
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                "kernels": kern}
    if dom == "residual":
        # the FP64 residual is kept in FP64 on purpose; on GB300 its limit is
        # the FP64 pipe (ncu capture of the V-cycle kernels at 1025^2)
        roofline["limiter"] = "FP64 pipe, 77 % busy in the ncu capture (6 FP64 operations per node)"

    # end to end through the C ABI with host buffers (pinned), the same steps
    e2e = None
    if not args.no_e2e:
        sim_e, io = timed_run(mixed_cfg, host_io=True, net=net, history=H, tune=TUNE)
        sim_e.close()
        e2e = {"value": job_value(io), "unit": "sim_yr/hr",
               "h2d_bytes_per_step": 8 * (4 * prob.nz + prob.ni * prob.nk),
               "d2h_bytes_per_step": 8 * (5 * prob.nz + prob.ni * prob.nk),
               "ms_per_step": io["ms"] / args.steps}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r = run_cpu(prob, args.warmup, args.steps, budget_s=args.cpu_sample_s)
        cpu = {"value": r["value"], "unit": "sim_yr/hr", "cores": r["threads"], "kind": "port",
               "sample": f"oracle (reference algorithm, {r['schedule']}): accepted steps "
                         f"{args.warmup + 1}..{args.warmup + r['steps']} from steady sliding, "
                         f"{r['wall_s']:.1f}s"}

    if rank == 0:
        guess = f"solution-history guess (last {H} solutions)" if H >= 2 else "previous-solution start"
        tn = head["autotune"]
        sched = (tn["nu_pre"], tn["nu_post"]) if tn else (mixed_cfg.nu_pre, mixed_cfg.nu_post)
        if tn:
            guess += f", autotuned tiles ({tn['box_down']}/{tn['box_up']}-column boxes)"
        else:
            guess += ", default 64-column tiles"
        mode = (f"learned warm start on the {guess} + FP32 cycles in FP64 refinement" if learned
                else f"{guess} + FP32 cycles in FP64 refinement")
        line = {
            "metric": METRIC, "value": value, "unit": "sim_yr/hr", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64+f32+bf16" if learned else "f64+f32", "data": "synthetic",
            "config": {"workload": f"{cfg.name}: {cfg.ni}x{cfg.nk} earthquake cycle, accepted RK43 steps "
                                   f"{args.warmup + 1}..{args.warmup + args.steps} from steady sliding",
                       "mg": f"{cfg.mg.n_levels} levels V({sched[0]},{sched[1]}), "
                             f"rel {cfg.mg.tol:g}, {mode}, exact coarsest solve, surface-row prolongation",
                       "parallelism": f"replicas x{world}", "l2": "flushed before every timed step"},
            "sim_years_timed": head["yrs"], "t_start_s": head["t0"], "t_end_s": head["t_end"],
            "vcycles_per_solve": head["vcycles"] / max(1, head["solves"]),
            "network_corrected_solves": head["net_solves"] / max(1, head["solves"]) if learned else None,
            "attempts_per_step": head["attempts"] / args.steps,
            "autotune": head["autotune"],
            **extra,
            "plain_fp64": None if plain is None else {
                "value": plain_value, "ms_per_step": plain["ms"] / args.steps,
                "vcycles_per_solve": plain["vcycles"] / max(1, plain["solves"]),
                "mg": "reference prolongation (no surface-row correction)"},
            "fp64_surface_prolong": None if plain_s is None else summary(plain_s),
            "speedup_vs_plain_fp64": value / world / plain_value if plain_value else None,
            "gpu_launches": head["launches"],
            "roofline": roofline, "clocks": clk, "e2e": e2e, "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if net is not None:
        net.close()
    sim.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
