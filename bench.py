#!/usr/bin/env python
"""Benchmark: simulated years per wall-hour of the quasi-dynamic earthquake
cycle at 1025 x 1025 (config 1 physics: layered mu, +-5% a-b perturbation,
8-level multigrid, 1e-9 relative residual; 365.25-day years).

A "step" is one accepted adaptive-RK43 step: the ARK4(3)6L stages, each an
elliptic multigrid solve plus the fault stress / Newton / aging-law update,
retried until the error test passes, then the refresh solve at the new state.

Every arm starts from the same fault-state checkpoint (the commit's refresh
solve from the zero-interior guess, then W untimed warm-up steps) and times
the same K accepted steps.  The default window is the plateau of config 1's
third rupture (``config1_1025_rupture3``: max V ~ 0.3 m/s, dt ~ 1.7e-2 s),
where about 70 % of a cycle's ~1,900 accepted steps are taken; dt is nearly
constant there, so the rate does not depend on W.  value = simulated years
advanced in the timed steps / their device time in hours.

The cycle-scale rate is measured beside it (``cycle``): one full earthquake
cycle -- 50 simulated years from the loading-phase checkpoint
``config1_1025_interseismic3`` (t = 100.2 yr), through the fourth rupture at
139.5 yr and its post-seismic phase -- for the GPU solvers.

Arms:
  default           this library on the GPU: the learned warm start with FP32
                    V-cycles in FP64 refinement (the headline); the same
                    solver without the network, FP64 variants and the plain
                    FP64 drop-in (the reference's algorithm) on the same steps
  --impl reference  the reference algorithm on the host cores (the CPU
                    oracle restating odeSolver.cpp / fault.cpp: 6 levels,
                    V(32,32)), same checkpoint, same W and K; beside it
                    (reference_gpu) the reference's own GPU path: its CUDA
                    kernels for every solve, host RK43 and fault code

The U-Net of the learned warm start is trained online first, on a separate
instance of the workload (the a-b perturbation drawn with the next seed):
config 3's protocol, the first 50 simulated years from steady sliding with
one Adam step per stage solve.

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
# 1025^2 and the U-Net's first 16 -> 16 channel convolution on the network's
# grid, keyed by the network's nodes per side
TRAFFIC = {"up0": 31.19e6, "down0": 17.35e6, "residual": 33.90e6}
TRAFFIC_CONV16 = {513: 8.62e6, 1025: 34.03e6}
METRIC = "simulated yr/hr at 1025² (learned+mixed vs plain FP64 MG, 1e-9 rel residual)"
WINDOW = "config1_1025_rupture3"
CYCLE_START = "config1_1025_interseismic3"
CYCLE_YEARS = 50.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", default="config1")
    p.add_argument("--window", default=WINDOW, help="fault-state checkpoint the timed steps start from")
    p.add_argument("--cpu-sample-s", type=float, default=20.0,
                   help="cpu_baseline leg: stop timing after the step that passes this many seconds")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-ref-gpu", action="store_true",
                   help="--impl reference: skip the reference's own GPU multigrid path")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cycle", action="store_true", help="skip the full-cycle runs")
    p.add_argument("--cycle-plain", action="store_true",
                   help="also run the plain FP64 drop-in (the reference's algorithm) through the full "
                        "cycle (about 2.5 minutes)")
    p.add_argument("--no-hbm", action="store_true", help="skip the 4097^2 HBM roofline of the V-cycle kernels")
    p.add_argument("--hbm-only", action="store_true",
                   help="only the 4097^2 level-0 kernel timings (for profilers)")
    p.add_argument("--hbm-reps", type=int, default=50)
    p.add_argument("--no-ensemble", action="store_true")
    p.add_argument("--ensemble-only", action="store_true", help="only the ensemble measurement")
    p.add_argument("--ensemble-full", action="store_true",
                   help="config 4's full mix (256 instances) instead of the 20-instance miniature")
    p.add_argument("--headline-only", action="store_true",
                   help="time only the headline solver (no FP64 comparison, e2e, cycle or CPU runs)")
    p.add_argument("--train-years", type=float, default=50.0,
                   help="simulated years of online training from steady sliding on a separate instance "
                        "(config 3's protocol: the first 50 years)")
    p.add_argument("--train-steps", type=int, default=0,
                   help="train for this many accepted steps instead of --train-years")
    p.add_argument("--no-learned", action="store_true", help="headline without the learned warm start")
    p.add_argument("--lr", type=float, default=1e-3)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--profile-run", action="store_true",
                   help="only the headline solver's W + K steps (network trained first), for per-kernel "
                        "profilers; prints a one-line summary")
    p.add_argument("--autotune", action="store_true",
                   help="qd_autotune the single-instance runs with the history guess after their warm-up "
                        "(by default they keep the config's V(2,2) and the default tiles)")
    p.add_argument("--no-autotune", action="store_true",
                   help="no tuning anywhere, the ensemble's instances included")
    p.add_argument("--schedule", default=None, help="nu_pre,nu_post of the fast runs (no tuning of them)")
    p.add_argument("--net-gate", type=float, default=0.0,
                   help="the network corrects a stage solve's guess when the guess's residual exceeds "
                        "this multiple of the solve's threshold (0: the measured rule, see --net-cost)")
    p.add_argument("--net-cost", type=float, default=2.0,
                   help="with --net-gate 0: the network's cost in V-cycles; it corrects guesses that would need "
                        "more than 1 + cost cycles")
    p.add_argument("--unet-level", type=int, default=1, choices=[0, 1, 2],
                   help="multigrid level whose grid the U-Net runs on (1: every other node, its "
                        "prediction prolongated bilinearly)")
    p.add_argument("--history", type=int, default=4,
                   help="stored solutions of the solution-history guess (0: start every solve "
                        "from the previous solution, as the reference)")
    p.add_argument("--newton-start", type=int, default=1, choices=[0, 1],
                   help="Newton start of the fast solvers (1: a binary32 solve of the log form, then the "
                        "reference's FP64 iteration; 0: the reference's x = 0); the plain FP64 drop-in and "
                        "the FP64 reference of the error measurement keep 0")
    p.add_argument("--tail-sweeps", type=int, default=1,
                   help="pre- and post-sweeps on the coarse tail's levels (<= 65 rows) of the fast solvers "
                        "(0: the fine levels' schedule); the plain FP64 drop-in and the FP64 reference of "
                        "the error measurement keep 0")
    p.add_argument("--smooth-ratio", type=float, default=2.5,
                   help="mixed-precision solvers: a level-0 smoothing pass instead of a V-cycle after a cycle "
                        "that left ||r|| within this ratio of the threshold (0: off)")
    p.add_argument("--config2-wall-s", type=float, default=240.0,
                   help="--config config2: seconds of stepping from steady sliding")
    p.add_argument("--error-steps", type=int, default=10,
                   help="fixed steps of the error-against-FP64 comparison")
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


def window_name(args, ck):
    m = ck["meta"]
    return (f"{m['config']}: {m['ni']}x{m['nk']} earthquake cycle from checkpoint {m['name']} "
            f"(t = {m['t_years']:.4f} yr, step {m['step']}, max V {m['max_V']:.3g} m/s), accepted RK43 steps "
            f"{m['step'] + args.warmup + 1}..{m['step'] + args.warmup + args.steps}")


# ---------------------------------------------------------------------------
# CPU arm: the reference algorithm through the oracle
# ---------------------------------------------------------------------------
def reference_mg_for(cfg):
    from qdeqcycle_fdm_gb300 import config
    r = config.reference_mg()
    r.tol_mode, r.tol = cfg.mg.tol_mode, cfg.mg.tol      # same accuracy target as the GPU arm
    r.max_cycles = 0
    return r


def run_cpu(prob, ck, warmup, steps, budget_s=None, gpu_multigrid=False):
    """Oracle RK43 from the checkpoint (refresh solve from the zero-interior
    guess): `warmup` untimed steps, then up to `steps` timed steps (stopping
    early once budget_s of timed work is spent, when given).  gpu_multigrid:
    every elliptic solve by the reference's own GPU kernels under its host
    sequencing (the reference program's split: host RK43 and fault code,
    GPU multigrid with u copied up and down every solve)."""
    import oracle
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    mg = reference_mg_for(prob.cfg)
    sim = oracle.Simulation(prob, mg.n_levels, mg.nu_pre, mg.nu_post, mg.nu_coarse, mg.tol_mode,
                            mg.tol, mg.max_cycles)
    rg = None
    if gpu_multigrid:
        rg = oracle.RefGpuMultigrid(prob, rel=mg.tol_mode, tol=mg.tol)
        rg.attach(sim)
    if sim.resume(ck) != 0:
        raise RuntimeError("the oracle's restart from the checkpoint failed")
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
    if rg is not None:
        rg.close()
    yrs = (s1["t"] - s0["t"]) / YEAR_S
    return {"value": yrs / (wall / 3600.0) if wall > 0 else 0.0, "wall_s": wall, "steps": n,
            "sim_years": yrs, "t_start_s": s0["t"], "t_end_s": s1["t"], "threads": threads,
            "vcycles_per_solve": (s1["vcycles"] - s0["vcycles"]) / max(1, s1["solves"] - s0["solves"]),
            "schedule": f"{mg.n_levels} levels V({mg.nu_pre},{mg.nu_post}), rel {mg.tol:g}"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from qdeqcycle_fdm_gb300 import checkpoints, config, problem
    import oracle
    oracle.build(ref=False)
    cfg = config.CONFIGS[args.config]()
    prob = problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])
    ck = checkpoints.load(args.window)
    r = run_cpu(prob, ck, args.warmup, args.steps)
    # the reference's GPU path: its own kernels for every solve (timed on the
    # same steps; the host RK43 / fault code stays on the CPU, as in the
    # reference program)
    if args.no_ref_gpu:
        ref_gpu = {"skipped": "--no-ref-gpu"}
    elif not oracle.refgpu_available():
        ref_gpu = {"unavailable": "oracle/_ref/ref_kernels.cubin or oracle/_build/librefgpu.so not built"}
    else:
        try:
            g = run_cpu(prob, ck, args.warmup, args.steps, gpu_multigrid=True)
            ref_gpu = {"value": g["value"], "unit": "sim_yr/hr", "ms_per_step": 1e3 * g["wall_s"] / max(1, g["steps"]),
                       "steps": g["steps"], "sim_years": g["sim_years"], "vcycles_per_solve": g["vcycles_per_solve"],
                       "what": "the reference's own CUDA kernels (odeSolver.cpp:757-1099, compiled unmodified) "
                               "under its host sequencing restated in C: 6 levels V(32,32), u up/down every solve, "
                               "a blocking cublasDnrm2 per V-cycle; host RK43 and fault code on "
                               f"{g['threads']} cores; same checkpoint, warm-up and steps"}
        except Exception as e:          # no GPU, or the driver refused
            ref_gpu = {"unavailable": f"{type(e).__name__}: {e}"}
    line = {
        "impl": "reference", "metric": METRIC, "value": r["value"], "unit": "sim_yr/hr",
        "n_gpus": args.gpus, "steps": r["steps"], "warmup": args.warmup,
        "ms_per_step": 1e3 * r["wall_s"] / max(1, r["steps"]), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": window_name(args, ck), "mg": r["schedule"], "l2": "host run",
                   "span_s": [r["t_start_s"], r["t_end_s"]]},
        "sim_years_timed": r["sim_years"],
        "cpu_baseline": {"value": r["value"], "unit": "sim_yr/hr", "cores": r["threads"], "kind": "port",
                         "sample": f"{r['steps']} accepted steps after {args.warmup} warm-up steps from "
                                   f"checkpoint {args.window}"},
        "e2e": {"value": r["value"], "unit": "sim_yr/hr", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "vcycles_per_solve": r["vcycles_per_solve"],
        "reference_gpu": ref_gpu,
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import numpy as np
    import torch

    from qdeqcycle_fdm_gb300 import api, build, checkpoints, config, problem, replicas, warmstart
    rank, world, local = replicas.env()
    torch.cuda.set_device(local)
    replicas.init("nccl")          # replicas only: the data path has no collective
    build.build()
    cfg = config.CONFIGS[args.config]()
    prob = problem.build_problem(cfg)            # face moduli homogenised on the GPU
    ck = checkpoints.load(args.window)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    H = args.history
    kslice = slice(1, prob.nk + 1)

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
        physics with another seed of the a-b perturbation): from steady
        sliding for --train-years simulated years (or --train-steps accepted
        steps), one Adam step per stage solve.  The timed runs then use the
        network on the benchmark instance, whose states it has not seen."""
        tcfg = cfg.replace(seed=cfg.seed + 1)
        tprob = problem.build_problem(tcfg)
        tsim = api.Simulation(tprob, mg)
        tsim.solver.set_solution_history(H)
        tsim.solver.set_newton_start(args.newton_start)
        tsim.solver.set_tail_sweeps(args.tail_sweeps)
        tsim.solver.set_smooth_correction(args.smooth_ratio)
        net = warmstart.UNet(unet_n(tprob.nk), unet_n(tprob.ni), seed=args.seed)
        net.attach(tsim.solver, warmstart.MODE_TRAIN, args.lr)
        tsim.start()
        w0 = time.perf_counter()
        if args.train_steps > 0:
            tsim.step(args.train_steps)
        else:
            while tsim.solver.rk43_state()["t"] < args.train_years * YEAR_S:
                tsim.step(50)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        st = tsim.state(with_u=False)
        n, loss = net.stats()
        net.attach(tsim.solver, warmstart.MODE_OFF)
        tsim.close()
        return net, {"train_samples": n, "last_loss": loss, "train_instance_seed": tcfg.seed,
                     "train_years": st["t"] / YEAR_S, "train_steps": st["it"], "train_wall_s": wall}

    def resumed(mg, history=0, net=None, start=None, params=None, newton=None, tail=None):
        """A solver restarted from a checkpoint (the window's by default);
        newton: the Newton start (default --newton-start), tail: the coarse
        tail's sweeps (default --tail-sweeps)."""
        sim = api.Simulation(prob, mg)
        sim.solver.set_solution_history(history)
        sim.solver.set_newton_start(args.newton_start if newton is None else newton)
        sim.solver.set_tail_sweeps(args.tail_sweeps if tail is None else tail)
        if mg.precision == 1:
            sim.solver.set_smooth_correction(args.smooth_ratio)
        if net is not None:
            net.attach(sim.solver, warmstart.MODE_PREDICT)
            warmstart.UNet.set_gate(sim.solver, args.net_gate)
            if args.net_gate == 0.0:
                warmstart.UNet.set_cost(sim.solver, args.net_cost)
        sim.resume(ck if start is None else start, params=params)
        return sim

    def timed_run(mg, host_io=False, net=None, history=0, tune=False, newton=None, tail=None):
        """Restart from the window checkpoint, W untimed warm-up steps, then
        K steps each bracketed by CUDA events on the solver's stream (L2
        flushed before each); with `history` >= 2 every stage solve starts
        from the solution-history guess, and with `net` from the network's
        correction of that guess; `tune`: qd_autotune on the run's own state
        after the warm-up steps (outside the timed region).  host_io: every
        step goes through the C ABI with host buffers -- state and u uploaded
        from pinned memory before, read back after (the e2e measurement)."""
        sim = resumed(mg, history, net, newton=newton, tail=tail)
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
        if args.profile_run:
            torch.cuda.profiler.start()   # ncu --profile-from-start off: capture the timed steps only
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if host_io:
                # the state and u in pinned host buffers, uploaded, stepped and
                # read back by one C-ABI call (qd_rk43_step_host)
                sim.solver.rk43_step_host(1, st, hU)
            else:
                sim.step(1)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            ms += step_ms[-1]
        if args.profile_run:
            torch.cuda.profiler.stop()
        barrier()
        s1 = sim.state(with_u=False)
        if net is not None:
            net.attach(sim.solver, warmstart.MODE_OFF)
        return sim, {"ms": ms, "yrs": (s1["t"] - s0["t"]) / YEAR_S, "step_ms": step_ms,
                     "t0": s0["t"], "t_end": s1["t"], "it0": s0["it"], "it1": s1["it"],
                     "launches": s1["kernel_launches"] - s0["kernel_launches"],
                     "vcycles": s1["vcycles"] - s0["vcycles"], "solves": s1["solves"] - s0["solves"],
                     "smooths": s1["smooth_corrections"] - s0["smooth_corrections"],
                     "newton": (s1["newton_iters"] - s0["newton_iters"]) / max(1, (s1["solves"] - s0["solves"]) * prob.nk),
                     "net_solves": s1["net_solves"] - s0["net_solves"],
                     "net_armed": s1["net_armed_solves"] - s0["net_armed_solves"],
                     "net_needed": s1["net_cycles_needed"] - s0["net_cycles_needed"],
                     "net_taken": s1["net_cycles_taken"] - s0["net_cycles_taken"],
                     "attempts": s1["attempts"] - s0["attempts"], "autotune": tuning}

    def job_value(run):
        """whole-job simulated yr/hr: years of all replicas / slowest rank's hours"""
        return replicas.aggregate(run["yrs"], run["ms"] / 3.6e6, device="cuda")[2]

    def reduce_max(x):
        return replicas.aggregate(0.0, x, device="cuda")[1]

    def summary(run):
        return {"value": job_value(run), "ms_per_step": reduce_max(run["ms"]) / args.steps,
                "vcycles_per_solve": run["vcycles"] / max(1, run["solves"]),
                "smoothing_passes_per_solve": run["smooths"] / max(1, run["solves"]),
                "solves_per_step": run["solves"] / args.steps, "sim_years_timed": run["yrs"],
                "newton_iters_per_node_solve": run["newton"],
                "span_s": [run["t0"], run["t_end"]]}

    def ensemble_run(ksteps=8, full=False):
        """Config 4's mix -- 96 x 257^2 + 96 x 513^2 + 64 x 1025^2 seeded
        instances (each its own parameters and adaptive dt) with full=True, or
        in miniature (12 + 6 + 2) -- advanced by qd_ensemble_step (GPU work of
        all instances interleaved) and, for comparison (miniature only), one
        instance after the other.  Host wall clock with the device synchronised
        on both sides (one stream per instance).  From steady sliding, after 3
        warm-up steps: the instances' dt ramps up from ini_dt, so the
        instance-years of the window say little; accepted instance-steps per
        second is the rate that does not depend on the window."""
        sizes = ([257] * 96 + [513] * 96 + [1025] * 64) if full else ([257] * 12 + [513] * 6 + [1025] * 2)
        cfgs = [config.ensemble_instance(n, i) for i, n in enumerate(sizes)]
        probs = [problem.build_problem(c) for c in cfgs]
        out = {"instances": ("96 x 257^2 + 96 x 513^2 + 64 x 1025^2" if full else
                             "12 x 257^2 + 6 x 513^2 + 2 x 1025^2") + " (config-4 parameter draws)",
               "steps_timed": ksteps, "warmup": 3, "history": H,
               "autotune": "per instance" if TUNE_ENSEMBLE else None}
        for mode in (("batched",) if full else ("batched", "sequential")):
            sims = [api.Simulation(p, c.mg) for p, c in zip(probs, cfgs)]
            for x in sims:
                x.solver.set_solution_history(H)
                x.solver.set_newton_start(args.newton_start)
                x.solver.set_tail_sweeps(args.tail_sweeps)
                x.solver.set_smooth_correction(args.smooth_ratio)
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
                         "instance_steps_per_s": len(sims) * ksteps / wall,
                         "instance_years_per_hr": yrs / (wall / 3600.0)}
            for x in sims:
                x.close()
        if not full:
            out["batched_speedup"] = out["sequential"]["wall_s"] / out["batched"]["wall_s"]
        return out

    if args.ensemble_only:
        if rank == 0:
            print(json.dumps({"ensemble": ensemble_run(full=args.ensemble_full)}), flush=True)
        return 0

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
                              "window": args.window, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": run["ms"] / args.steps,
                              "vcycles_per_solve": run["vcycles"] / max(1, run["solves"]),
                              "smoothing_passes_per_solve": run["smooths"] / max(1, run["solves"]),
                              "solves_per_step": run["solves"] / args.steps,
                              "network_corrected_solves": run["net_solves"] / max(1, run["solves"]),
                              "launches_per_step": run["launches"] / args.steps,
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
            "protocol": (f"trained online for {args.train_steps} accepted steps" if args.train_steps > 0 else
                         f"trained online over the first {args.train_years:g} simulated years from steady "
                         "sliding (config 3)") + " on a separate instance, one Adam step per stage solve",
            **tinfo, "lr": args.lr,
            "inference_us": us_f, "inference_tflops": fl_f / (us_f * 1e-6) / 1e12,
            "train_step_us": us_t, "train_tflops": fl_t / (us_t * 1e-6) / 1e12,
            "tensor_peak_tflops": bf, "inference_frac_of_peak": fl_f / (us_f * 1e-6) / 1e12 / bf}
    plain = plain_value = None
    if not args.headline_only:
        if H >= 2:
            simp, prev = timed_run(mixed_cfg)
            simp.close()
            extra["mixed_previous_solution_start"] = summary(prev)
            simh, fh = timed_run(fp64s_cfg, history=H)
            simh.close()
            extra["fp64_history"] = summary(fh)
        sim64, plain = timed_run(fp64_cfg, newton=0, tail=0)
        sim64.close()
        sim64s, plain_s = timed_run(fp64s_cfg)
        sim64s.close()
        extra["fp64_surface_prolong"] = summary(plain_s)
        plain_value = plain["yrs"] / (reduce_max(plain["ms"]) / 3.6e6)

    # --- error of the headline against FP64, identical fixed steps ---------
    def error_vs_fp64(nsteps):
        """From the window checkpoint, `nsteps` steps of the checkpoint's dt
        (fixed) with the headline solver and with FP64 V-cycles solved to a
        1e-12 relative residual (the drop-in's FP64 arithmetic, held to the
        CPU oracle by the parity tests); also FP64 at the headline's 1e-9, to
        show what that tolerance alone lets through.  Max relative errors:
        u and tau, slip, psi against the field's max |.|, V node by node."""
        dt = ck["dt"]
        params = (prob.tmax, dt, dt, dt, prob.totTol, 2**31 - 1)
        tight = config.MGConfig(**{**fp64s_cfg.__dict__, "tol": 1e-12, "max_cycles": 400})
        runs = {}
        for name, mg, hist, nn in (("exact", tight, 0, None), ("fp64_1e-9", fp64s_cfg, 0, None),
                                   ("headline", mixed_cfg, H, net)):
            s = resumed(mg, hist, nn, params=params, newton=0 if name == "exact" else None,
                        tail=0 if name == "exact" else None)
            s.step(nsteps)
            runs[name] = s.state()
            if nn is not None:
                nn.attach(s.solver, warmstart.MODE_OFF)
            s.close()
        ex = runs["exact"]

        def errs(g):
            def rmax(a, b):
                return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
            return {"u": rmax(g["U"], ex["U"]),
                    "tau": rmax(g["Ts"][kslice] + prob.tau0[kslice], ex["Ts"][kslice] + prob.tau0[kslice]),
                    "V": float(np.max(np.abs(g["V"][kslice] - ex["V"][kslice]) / ex["V"][kslice])),
                    "slip": rmax(g["Slip"][kslice], ex["Slip"][kslice]),
                    "psi": rmax(g["psi"][kslice], ex["psi"][kslice])}
        return {"steps": nsteps, "dt_s": dt, "reference": "FP64 V(2,2) cycles to a 1e-12 relative residual",
                "headline": errs(runs["headline"]), "fp64_at_1e-9": errs(runs["fp64_1e-9"])}

    err = None if args.headline_only else error_vs_fp64(args.error_steps)

    # --- one full earthquake cycle ------------------------------------------
    def cycle_run(mg, history=0, nn=None):
        """From the loading-phase checkpoint to CYCLE_YEARS later (tmax): the
        whole span timed with CUDA events on the solver's stream, in calls
        of up to 200 accepted steps (no L2 flush inside: one timed region)."""
        cst = checkpoints.load(CYCLE_START)
        params = (cst["t"] + CYCLE_YEARS * YEAR_S, prob.ini_dt, prob.mindt, prob.maxdt, prob.totTol,
                  int(min(prob.maxNumSteps, 2**31 - 1)))
        s = resumed(mg, history, nn, start=cst, params=params)
        stream = torch.cuda.ExternalStream(s.solver.stream_ptr())
        s0 = s.state(with_u=False)
        vmax_hi = False
        ruptures = 0
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        w0 = time.perf_counter()
        while True:
            done = s.step(200)
            st = s.solver.rk43_state()
            hi = float(np.max(st["V"][kslice])) > 0.1
            ruptures += int(hi and not vmax_hi)
            vmax_hi = hi
            if done < 200:
                break
        e1.record(stream)
        e1.synchronize()
        wall = time.perf_counter() - w0
        ms = e0.elapsed_time(e1)
        s1 = s.state(with_u=False)
        if nn is not None:
            nn.attach(s.solver, warmstart.MODE_OFF)
        s.close()
        yrs = (s1["t"] - s0["t"]) / YEAR_S
        nst = s1["it"] - s0["it"]
        return {"value": yrs / (ms / 3.6e6), "sim_years": yrs, "steps": nst, "ms": ms, "ms_per_step": ms / nst,
                "host_wall_s": wall, "vcycles_per_solve": (s1["vcycles"] - s0["vcycles"]) / max(1, s1["solves"] - s0["solves"]),
                "smoothing_passes_per_solve": (s1["smooth_corrections"] - s0["smooth_corrections"])
                / max(1, s1["solves"] - s0["solves"]),
                "solves_per_step": (s1["solves"] - s0["solves"]) / nst,
                "network_corrected_solves": (s1["net_solves"] - s0["net_solves"]) / max(1, s1["solves"] - s0["solves"]),
                "network_armed_solves": (s1["net_armed_solves"] - s0["net_armed_solves"])
                / max(1, s1["solves"] - s0["solves"]),
                "network_cycles_needed_taken": [s1["net_cycles_needed"] - s0["net_cycles_needed"],
                                                s1["net_cycles_taken"] - s0["net_cycles_taken"]],
                "ruptures_seen": ruptures}

    cycle = None
    if not args.no_cycle and not args.headline_only:
        cycle = {"span": f"{CYCLE_YEARS:g} simulated years from checkpoint {CYCLE_START} "
                         "(loading phase, t = 100.2 yr) through the next rupture and its post-seismic phase",
                 "timing": "CUDA events around the whole span (no L2 flush inside)"}
        if learned:
            cycle["headline"] = cycle_run(mixed_cfg, H, net)
        cycle["mixed_no_learned"] = cycle_run(mixed_cfg, H)
        cycle["fp64_history"] = cycle_run(fp64s_cfg, H)
        if args.cycle_plain:
            cycle["plain_fp64"] = cycle_run(fp64_cfg)

    if not args.headline_only and not args.no_ensemble:
        extra["ensemble"] = ensemble_run(full=args.ensemble_full)

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
    #   residual FP64 u and the moduli cx, cz, diag (double-float pairs)
    #            read + FP32 rhs written: 36 B per node
    #   conv16   16 BF16 channels read and written: 64 B per padded pixel of
    #            the network's grid
    # Launches per step: one of each cycle kernel per V-cycle, the residual
    # once more per solve (the guess) and once more per solve the network
    # corrected, the convolution 4 per corrected solve.  The dominant kernel
    # (largest time x launches per step) is the roofline entry.  At 1025^2
    # the V-cycle's arrays stay in the 129 MB L2 between back-to-back
    # launches, so these are effective rates; the same kernels at 4097^2
    # (arrays of 67 MB each per FP32 field) give the HBM fractions.
    peak = peaks.get("hbm_gbs", 6800.0)
    tn = head["autotune"]
    nu_pre, nu_post = (tn["nu_pre"], tn["nu_post"]) if tn else (mixed_cfg.nu_pre, mixed_cfg.nu_post)

    def algo_bytes(ni, nk):
        n0 = ni * nk
        n1 = ((ni - 1) // 2 + 1) * ((nk - 1) // 2 + 1)
        return {"up0": (24.0 + 20.0 * nu_post) * n0 + 4.0 * n1, "down0": (16.0 + 20.0 * nu_pre) * n0 + 4.0 * n1,
                "residual": 36.0 * n0}

    # the network's padded grid (H+2 rows x W+2 columns rounded up to 8)
    pad_px = (unet_n(cfg.nk) + 2) * ((unet_n(cfg.ni) + 2 + 7) // 8 * 8)
    algo = {**algo_bytes(cfg.ni, cfg.nk), "conv16": 64.0 * pad_px}
    names = {"up0": f"k_up<float,2> level 0 (prolongation + {nu_post} sweep(s) + u64 += e)",
             "down0": f"k_down<float> level 0 ({nu_pre} sweep(s) + residual + restriction)",
             "residual": "k_residual_df (level-0 residual in double-float -> FP32 rhs + norm)",
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
                "grid": "1025x1025 (L2-resident between launches: effective rate)",
                "kernels": kern}
    if not args.no_hbm:
        roofline["hbm_4097"] = hbm_kernels(api, config, problem, mixed_cfg, algo_bytes, names, peak, REPS)

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
        r = run_cpu(prob, ck, args.warmup, args.steps, budget_s=args.cpu_sample_s)
        cpu = {"value": r["value"], "unit": "sim_yr/hr", "cores": r["threads"], "kind": "port",
               "sample": f"oracle (reference algorithm, {r['schedule']}): accepted steps "
                         f"{ck['it'] + args.warmup + 1}..{ck['it'] + args.warmup + r['steps']} from checkpoint "
                         f"{args.window}, {r['wall_s']:.1f}s",
               "ms_per_step": 1e3 * r["wall_s"] / max(1, r["steps"])}

    if rank == 0:
        guess = f"solution-history guess (last {H} solutions)" if H >= 2 else "previous-solution start"
        tn = head["autotune"]
        sched = (tn["nu_pre"], tn["nu_post"]) if tn else (mixed_cfg.nu_pre, mixed_cfg.nu_post)
        if tn:
            guess += f", autotuned tiles ({tn['box_down']}/{tn['box_up']}-column boxes)"
        else:
            guess += ", default tiles (96-column k_down and 64-column k_up boxes at level 0)"
        mode = (f"learned warm start on the {guess} + FP32 cycles in FP64 refinement" if learned
                else f"{guess} + FP32 cycles in FP64 refinement")
        line = {
            "metric": METRIC, "value": value, "unit": "sim_yr/hr", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64+f32+bf16" if learned else "f64+f32", "data": "synthetic",
            "config": {"workload": window_name(args, ck),
                       "span_s": [head["t0"], head["t_end"]],
                       "mg": f"{cfg.mg.n_levels} levels V({sched[0]},{sched[1]}), "
                             f"rel {cfg.mg.tol:g}, {mode}, exact coarsest solve, surface-row prolongation",
                       "newton_start": ("binary32 log-form solve, then the reference's FP64 iteration"
                                        if args.newton_start else "the reference's x = 0"),
                       "tail_sweeps": (f"V({args.tail_sweeps},{args.tail_sweeps}) on the levels of <= 65 rows"
                                       if args.tail_sweeps else "the fine schedule on every level"),
                       "parallelism": f"replicas x{world}", "l2": "flushed before every timed step"},
            "sim_years_timed": head["yrs"], "t_start_s": head["t0"], "t_end_s": head["t_end"],
            "vcycles_per_solve": head["vcycles"] / max(1, head["solves"]),
            "smoothing_passes_per_solve": head["smooths"] / max(1, head["solves"]),
            "solves_per_step": head["solves"] / args.steps,
            "newton_iters_per_node_solve": head["newton"],
            "network_corrected_solves": head["net_solves"] / max(1, head["solves"]) if learned else None,
            "network_armed_solves": head["net_armed"] / max(1, head["solves"]) if learned else None,
            "network_gate": (f"measured: corrects guesses that would need more than {1 + args.net_cost:g} V-cycles"
                             if args.net_gate == 0.0 else f"fixed: ||r|| > {args.net_gate:g} x threshold")
            if learned else None,
            "network_cycles_needed_taken": [head["net_needed"], head["net_taken"]] if learned else None,
            "attempts_per_step": head["attempts"] / args.steps,
            "autotune": head["autotune"],
            "error_vs_fp64": err,
            "cycle": cycle,
            **extra,
            "plain_fp64": None if plain is None else {
                "value": plain_value, "ms_per_step": plain["ms"] / args.steps,
                "vcycles_per_solve": plain["vcycles"] / max(1, plain["solves"]),
                "newton_iters_per_node_solve": plain["newton"],
                "mg": "the reference's algorithm: prolongation without the surface row, coarsest-level sweeps, "
                      "previous-solution start, Newton from x = 0, the fine schedule on every level"},
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


def hbm_kernels(api, config, problem, mixed_cfg, algo_bytes, names, peak, reps):
    """The level-0 V-cycle kernels on a 4097 x 4097 grid of config 1's
    physics (10 levels): each FP32 field is 67 MB, the tile kernels' five
    staged arrays 335 MB, so back-to-back launches stream from HBM.  Timed
    like the 1025^2 kernels (REPS launches between CUDA events) on a field
    of seeded random values with the boundary columns set."""
    import numpy as np
    cfg = config.config1().replace(ni=4097, nk=4097, name="config1_4097")
    prob = problem.build_problem(cfg)
    mg = config.MGConfig(**{**mixed_cfg.__dict__, "n_levels": 10})
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, mg)
    rng = np.random.default_rng(5)
    U = np.zeros((prob.nz, prob.nx))
    U[1:-1, 1:-1] = rng.normal(size=(prob.nk, prob.ni)) * 1e-3
    U[1:-1, 1] = 1.0
    s.upload_u(U)
    ab = algo_bytes(cfg.ni, cfg.nk)
    out = {"grid": "4097x4097 (config 1 physics, 10 levels; arrays larger than L2: HBM rate)", "kernels": {}}
    for k in ("down0", "up0", "residual"):
        s.time_kernel(k, 3)
        us = s.time_kernel(k, reps)
        gbs = ab[k] / (us * 1e-6) / 1e9
        out["kernels"][k] = {"kernel": names[k], "us": us, "algo_bytes": ab[k], "achieved_gbs": gbs,
                             "frac": gbs / peak}
    s.close()
    return out


def run_config2(args):
    """Config 2 (4097^2 stretched in depth, FP32 V(2,2) cycles in FP64
    refinement to 1e-9, solution-history guess): from steady sliding for
    --config2-wall-s seconds of GPU time (or config 2's 100 simulated years,
    whichever comes first), reporting simulated years per hour, steps,
    V-cycles per solve and ruptures; then the error of the mixed solver
    against FP64 V-cycles solved to 1e-12 on 5 identical fixed steps from
    the state reached, and the level-0 kernels' HBM roofline on this grid.
    Prints one JSON line (not the headline contract's)."""
    import numpy as np
    import torch

    from qdeqcycle_fdm_gb300 import api, build, checkpoints, config, problem
    build.build()
    cfg = config.config2()
    t0 = time.perf_counter()
    prob = problem.build_problem(cfg)
    setup_s = time.perf_counter() - t0
    k = slice(1, prob.nk + 1)
    sim = api.Simulation(prob, cfg.mg)
    sim.solver.set_solution_history(args.history)
    sim.solver.set_newton_start(args.newton_start)
    sim.solver.set_tail_sweeps(args.tail_sweeps)
    sim.solver.set_smooth_correction(args.smooth_ratio)
    sim.start()
    stream = torch.cuda.ExternalStream(sim.solver.stream_ptr())
    s0 = sim.state(with_u=False)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    w0 = time.perf_counter()
    hi, ruptures, vmax = False, 0, 0.0
    rck = None        # a state inside the last rupture (20 calls after its onset), for the error check
    since = -1
    while time.perf_counter() - w0 < args.config2_wall_s:
        done = sim.step(10)
        st = sim.solver.rk43_state()
        v = float(np.max(st["V"][k]))
        vmax = max(vmax, v)
        if v > 0.1 and not hi:
            ruptures += 1
            since = 0
        hi = v > 0.1
        if since >= 0:
            since += 1
            if since == 20 and hi:
                rck = (checkpoints.from_state(st), sim.solver.download_u(), v)
        if done < 10:
            break
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    s1 = sim.state(with_u=False)
    yrs = (s1["t"] - s0["t"]) / YEAR_S
    nst = s1["it"] - s0["it"]
    if rck is not None:
        ck, U, v_ck = rck
    else:
        ck, U, v_ck = checkpoints.from_state(st), sim.solver.download_u(), v
    sim.close()
    run = {"sim_years": yrs, "steps": nst, "ms": ms, "ms_per_step": ms / max(1, nst),
           "value": yrs / (ms / 3.6e6), "vcycles_per_solve": (s1["vcycles"] - s0["vcycles"]) / max(1, s1["solves"] - s0["solves"]),
           "smoothing_passes_per_solve": (s1["smooth_corrections"] - s0["smooth_corrections"])
           / max(1, s1["solves"] - s0["solves"]),
           "ruptures_seen": ruptures, "max_V": vmax, "t_end_yr": s1["t"] / YEAR_S, "dt_end_s": s1["dt"]}

    # error against FP64 on identical fixed steps from the state reached
    dt = ck["dt"]
    params = (prob.tmax, dt, dt, dt, prob.totTol, 2**31 - 1)
    tight = config.MGConfig(**{**cfg.mg.__dict__, "precision": 0, "tol": 1e-12, "max_cycles": 400})
    fp64 = config.MGConfig(**{**cfg.mg.__dict__, "precision": 0})
    out = {}
    for name, mg, hist in (("exact", tight, 0), ("fp64_1e-9", fp64, 0), ("mixed", cfg.mg, args.history)):
        x = api.Simulation(prob, mg)
        x.solver.set_solution_history(hist)
        x.solver.set_newton_start(args.newton_start if name == "mixed" else 0)
        x.solver.set_tail_sweeps(args.tail_sweeps if name == "mixed" else 0)
        if name == "mixed":
            x.solver.set_smooth_correction(args.smooth_ratio)
        x.resume(ck, U=U, params=params)
        x.step(5)
        out[name] = x.state()
        x.close()
    ex = out["exact"]

    def errs(g):
        def rmax(a, b):
            return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
        return {"u": rmax(g["U"], ex["U"]), "tau": rmax(g["Ts"][k] + prob.tau0[k], ex["Ts"][k] + prob.tau0[k]),
                "V": float(np.max(np.abs(g["V"][k] - ex["V"][k]) / ex["V"][k])),
                "slip": rmax(g["Slip"][k], ex["Slip"][k]), "psi": rmax(g["psi"][k], ex["psi"][k])}
    err = {"steps": 5, "dt_s": dt, "from": f"t = {ck['t'] / YEAR_S:.4f} yr, max V {v_ck:.3g} m/s",
           "reference": "FP64 V(2,2) cycles to a 1e-12 relative residual",
           "mixed": errs(out["mixed"]), "fp64_at_1e-9": errs(out["fp64_1e-9"])}

    # level-0 kernels on this grid (arrays larger than L2)
    peak = _peaks().get("hbm_gbs", 6800.0)
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, cfg.mg, jrow=prob.jrow)
    s.upload_u(U)
    n0 = prob.ni * prob.nk
    n1 = ((prob.ni - 1) // 2 + 1) * ((prob.nk - 1) // 2 + 1)
    nu = cfg.mg.nu_pre
    ab = {"up0": (24.0 + 20.0 * nu) * n0 + 4.0 * n1, "down0": (16.0 + 20.0 * nu) * n0 + 4.0 * n1,
          "residual": 36.0 * n0}
    kern = {}
    for kk in ("down0", "up0", "residual", "tail"):
        s.time_kernel(kk, 3)
        us = s.time_kernel(kk, 50)
        kern[kk] = {"us": us}
        if kk in ab:
            gbs = ab[kk] / (us * 1e-6) / 1e9
            kern[kk].update(algo_bytes=ab[kk], achieved_gbs=gbs, frac=gbs / peak)
    s.close()
    print(json.dumps({"config": "config2_4097: 4097x4097 stretched in depth (4x finer rows over 0-20 km), "
                                "config 0 friction with Dc = 2 mm, mu 30 GPa, 10 levels V(2,2), FP32 cycles in "
                                "FP64 refinement to 1e-9 relative, solution-history guess",
                      "setup_s": setup_s, "run": run, "error_vs_fp64": err,
                      "hbm_roofline": {"peak_gbs": peak, "kernels": kern}}), flush=True)
    return 0


def run_hbm_only(args):
    """Only the level-0 V-cycle kernels on the 4097^2 grid (hbm_kernels), for
    profilers: 3 warm-up and --hbm-reps timed launches of each kernel."""
    from qdeqcycle_fdm_gb300 import api, build, config, problem
    build.build()
    mixed = config.MGConfig(**{**config.config1().mg.__dict__, "precision": 1, "surface_prolong": 1,
                               "coarse_solve": 1})
    n0, n1 = 4097 * 4097, 2049 * 2049

    def algo_bytes(ni, nk):
        return {"up0": (24.0 + 20.0 * mixed.nu_post) * n0 + 4.0 * n1,
                "down0": (16.0 + 20.0 * mixed.nu_pre) * n0 + 4.0 * n1, "residual": 36.0 * n0}
    names = {"down0": "k_down<float> level 0", "up0": "k_up<float,2> level 0",
             "residual": "k_residual_df"}
    peak = _peaks().get("hbm_gbs", 6800.0)
    print(json.dumps(hbm_kernels(api, config, problem, mixed, algo_bytes, names, peak, args.hbm_reps)), flush=True)
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
    if args.config == "config2":
        return run_config2(args)
    if args.hbm_only:
        return run_hbm_only(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
