"""The headline solver -- the learned correction on the solution-history
guess, FP32 V-cycles inside FP64 iterative refinement with the
double-float residual, the binary32 Newton start, V(1,1) on the coarse
tail and the level-0 smoothing pass -- against the CPU oracle's FP64 RK43
loop (the reference's Newton start and schedule) on identical fixed steps,
through a rupture.

A 257 x 257 problem with config 1's physics (layered medium, +-5 % a-b
perturbation) runs on the GPU from steady sliding into its first rupture
(one Adam step of the U-Net per stage solve on the way) until the slip rate
passes 0.1 m/s; its fault state there becomes the checkpoint both sides
resume from.  Then both take the same fixed steps, half the checkpoint's
adaptive dt (a fixed step must stay stable while the rupture accelerates):
the GPU with the network in
prediction mode and a gate that lets it correct every guess that misses the
tolerance, the oracle in plain FP64 solved to a 1e-12 relative residual
(the reference solution) and, for scale, at the headline's 1e-9.  Each solve
ends within its tolerance of the exact discrete solution; tau (a one-sided
derivative of u at the fault) and V (exponential in tau / (a sigma_n)) carry
that error amplified.  The headline must stay within 10x of what FP64 at
the same 1e-9 lets through, field by field, and within absolute bounds
(u 1e-7, tau 1e-6, V 1e-4, slip and psi 1e-7 relative).
"""
import numpy as np
import pytest

import oracle
from qdeqcycle_fdm_gb300 import api, checkpoints, config, problem, warmstart

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_learned_mixed_steps_through_a_rupture_match_fp64_oracle(gpu_lib, oracle_lib):
    import os
    oracle.set_threads(os.cpu_count() or 1)
    n = 257
    cfg = config.small(n, mu_profile="layered", amb_perturb=0.05)
    prob = problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])
    mg = config.MGConfig(n_levels=cfg.mg.n_levels, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1, tol=1e-9,
                         max_cycles=200, precision=1, surface_prolong=1, coarse_solve=1)
    # into the first rupture, training the network on the way
    sim = api.Simulation(prob, mg)
    sim.solver.set_solution_history(4)
    # the bench's headline settings: binary32 Newton start, V(1,1) on the
    # coarse tail's levels, the level-0 smoothing pass
    sim.solver.set_newton_start(1)
    sim.solver.set_tail_sweeps(1)
    sim.solver.set_smooth_correction(2.5)
    net = warmstart.UNet((n - 1) // 2 + 1, (n - 1) // 2 + 1, seed=3)
    net.attach(sim.solver, warmstart.MODE_TRAIN, 1e-3)
    sim.start()
    k = slice(1, prob.nk + 1)
    for _ in range(3000):
        sim.step(1)
        st = sim.solver.rk43_state()
        if np.max(st["V"][k]) > 0.1:
            break
    assert np.max(st["V"][k]) > 0.1, "no rupture within 3000 steps"
    trained, _ = net.stats()
    assert trained > 0
    ck = checkpoints.from_state(st)
    U0 = sim.solver.download_u()
    dt = 0.5 * ck["dt"]
    ck["dt"] = dt
    params = (prob.tmax, dt, dt, dt, prob.totTol, 2**31 - 1)

    # the same fixed steps: GPU headline (network predicting) vs FP64 oracle
    net.attach(sim.solver, warmstart.MODE_PREDICT)
    warmstart.UNet.set_gate(sim.solver, 1.0)
    sim.resume(ck, U=U0, params=params)
    nsteps = 20

    def oracle_run(tol):
        cpu = oracle.Simulation(prob, mg.n_levels, 2, 2, 32, 1, tol, 400, surface_prolong=1, coarse_solve=1)
        cpu.set_params(*params)
        assert cpu.resume(ck, U=U0) == 0
        for _ in range(nsteps):
            assert cpu.step() == 0
        return cpu.state()

    exact = oracle_run(1e-12)
    fp64 = oracle_run(1e-9)
    s0 = sim.solver.stats()
    sim.step(nsteps)
    s1 = sim.solver.stats()
    g = sim.state()
    net.attach(sim.solver, warmstart.MODE_OFF)
    net.close()
    sim.close()
    # the learned correction ran in these steps
    assert s1["net_solves"] > s0["net_solves"]
    assert g["it"] == exact["it"] == ck["it"] + nsteps
    assert rel(g["t"], exact["t"]) < 1e-15

    def errs(x):
        return {"u": rel(x["U"], exact["U"]),
                "tau": rel(x["Ts"][k] + prob.tau0[k], exact["Ts"][k] + prob.tau0[k]),
                "V": float(np.max(np.abs(x["V"][k] - exact["V"][k]) / exact["V"][k])),
                "slip": rel(x["Slip"][k], exact["Slip"][k]), "psi": rel(x["psi"][k], exact["psi"][k])}
    e_gpu, e_fp64 = errs(g), errs(fp64)
    msg = {"headline": e_gpu, "fp64_at_1e-9": e_fp64}
    bounds = {"u": 1e-7, "tau": 1e-6, "V": 1e-4, "slip": 1e-7, "psi": 1e-7}
    for key, b in bounds.items():
        assert e_gpu[key] < b, msg
        assert e_gpu[key] <= 10.0 * e_fp64[key] + 1e-13, msg
