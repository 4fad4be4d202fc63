"""The oracle's multigrid against the reference's own CUDA kernels.

Two pins:
  * ``ref_kernels_golden.npz`` -- outputs of the reference's kernels (compiled
    unmodified from odeSolver.cpp, run on a GB300 by
    tests/golden/make_golden_kernels.py); checked against the oracle on the
    CPU, so this pin needs no GPU;
  * live, on a GPU: the reference's kernels (oracle/_ref/ref_kernels.cubin),
    the oracle and this library's kernels on the same inputs.
The reference's kernels are built with nvcc's default FMA contraction; the
oracle rounds every operation, so agreement is to ~1e-13, not bit-exact.
"""
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "ref_kernels_golden.npz")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def gold(oracle_lib):
    if not os.path.exists(GOLD):
        pytest.skip("reference-kernel golden vectors not generated yet")
    return np.load(GOLD)


def _mg(g):
    return oracle.Multigrid(int(g["ni"]), int(g["nk"]), float(g["dh"]), g["mu_equi"], 6, 32, 32, 32)


def test_oracle_smooth_matches_reference_kernels(gold):
    mg = _mg(gold)
    u = gold["u0"].copy()
    f = np.zeros_like(u)
    for _ in range(32):
        mg.rbgs(u, f, 0, 0)
        mg.rbgs(u, f, 0, 1)
    assert rel(u, gold["smooth0"]) < 1e-13


def test_oracle_coarse_smooth_matches_reference_kernels(gold):
    mg = _mg(gold)
    e = gold["c_e_in"].copy()
    f = np.ascontiguousarray(gold["c_f"])
    for _ in range(32):
        mg.rbgs(e, f, 2, 0)
        mg.rbgs(e, f, 2, 1)
    assert rel(e, gold["c_smooth2"]) < 1e-12


def test_oracle_vcycle_matches_reference_kernels(gold):
    mg = _mg(gold)
    u = gold["u0"].copy()
    mg.vcycle(u, np.zeros_like(u))
    assert rel(u, gold["vcycle"]) < 1e-12


def test_oracle_multigrid_matches_reference_kernels(gold):
    mg = _mg(gold)
    u = gold["u0"].copy()
    cyc, rn, _ = mg.solve(u, tol_mode=0, tol=1e-9, max_cycles=1000)
    assert cyc == int(gold["mg_cycles"])
    assert rel(u, gold["mg_u"]) < 1e-11


@pytest.mark.gpu
def test_live_reference_kernels_vs_oracle_and_library(gpu_lib, oracle_lib):
    from oracle import refkernels
    if not refkernels.available():
        pytest.skip("oracle/_ref/ref_kernels.cubin not built (needs the reference sources)")
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden_kernels import inputs
    from qdeqcycle_fdm_gb300 import api, config
    prob, u0 = inputs()
    R = refkernels.RefKernels(prob.ni, prob.nk, prob.dh, prob.mu_equi)
    u = R.to_dev(u0)
    f = R.torch.zeros_like(u)
    R.vcycle(u, f, 0)
    ref_v = u.cpu().numpy().reshape(u0.shape)
    u = R.to_dev(u0)
    cyc_ref, _ = R.multigrid(u, f, 1e-9)
    ref_mg = u.cpu().numpy().reshape(u0.shape)
    R.close()
    mg = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, 6, 32, 32, 32)
    uo = u0.copy()
    mg.vcycle(uo, np.zeros_like(uo))
    assert rel(uo, ref_v) < 1e-12
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, config.reference_mg())
    U = np.zeros((prob.nz, prob.nx))
    U[1:-1, 1:-1] = u0
    s.upload_u(U)
    s.vcycle()
    assert rel(s.download_u()[1:-1, 1:-1], ref_v) < 1e-12
    s.upload_u(U)
    ref = config.reference_mg()
    ref.max_cycles = 1000
    s.set_options(ref)
    cyc, rn, _ = s.ode_solve()
    assert cyc == cyc_ref
    assert rel(s.download_u()[1:-1, 1:-1], ref_mg) < 1e-11


@pytest.mark.gpu
def test_reference_gpu_path_under_the_oracle_rk43(gpu_lib, oracle_lib):
    """The reference's GPU path as the bench's reference arm times it: the
    oracle's RK43 loop with every elliptic solve done by the reference's own
    kernels under its host sequencing (oracle/refgpu.c).  Three accepted
    steps on a 65^2 problem against the same loop solving on the CPU with
    the same schedule (6 levels V(32,32), relative 1e-10): same V-cycle
    counts, states to 1e-9 (the kernels contract multiply-adds, the oracle
    does not)."""
    if not oracle.refgpu_available():
        pytest.skip("oracle/_ref/ref_kernels.cubin not built (needs the reference sources)")
    from qdeqcycle_fdm_gb300 import config, problem
    cfg = config.small(65, mu_profile="layered", layer_depth_km=20.0)
    prob = problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])
    runs = []
    for gpu in (False, True):
        sim = oracle.Simulation(prob, 6, 32, 32, 32, 1, 1e-10, 0)
        rg = None
        if gpu:
            rg = oracle.RefGpuMultigrid(prob, rel=1, tol=1e-10)
            rg.attach(sim)
        sim.start()
        for _ in range(3):
            assert sim.step() == 0
        runs.append(sim.state())
        if rg is not None:
            st = rg.stats()
            assert st["solves"] == runs[-1]["solves"] and st["vcycles"] == runs[-1]["vcycles"]
            rg.close()
    cpu, gpu = runs
    k = slice(1, prob.nk + 1)
    assert gpu["vcycles"] == cpu["vcycles"]
    assert rel(gpu["U"], cpu["U"]) < 1e-9
    assert rel(gpu["V"][k], cpu["V"][k]) < 1e-9
    assert abs(gpu["t"] - cpu["t"]) <= 1e-12 * cpu["t"]
