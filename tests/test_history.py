"""Initial guess from the solution history (qd_set_solution_history).

The guess only moves the starting point of each stage solve, so:
  * with solves tight enough that the tolerance is not what differs, 100
    accepted RK43 steps with the history guess match the oracle (which starts
    every solve from the previous solution, as the reference) to the parity
    bar: u, tau, V to 1e-10 and slip, psi to 1e-8 relative;
  * at the bench's 1e-9 relative tolerance the same run needs fewer V-cycles
    per solve than with the previous-solution start, and its state stays
    within the tolerance's reach of that run (fixed steps, so that both runs
    visit the same times).
"""
import numpy as np
import pytest

import oracle
from qdeqcycle_fdm_gb300 import _lib, api, config, problem

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def make_problem(n, **kw):
    cfg = config.small(n, **kw)
    return cfg, problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])


@pytest.fixture(scope="module", autouse=True)
def _libs(gpu_lib, oracle_lib):
    return gpu_lib


def test_history_guess_keeps_oracle_parity():
    cfg, prob = make_problem(65)
    prob.ini_dt = prob.mindt = prob.maxdt = 3e5
    mg = config.MGConfig(n_levels=cfg.mg.n_levels, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1,
                         tol=1e-13, max_cycles=400, surface_prolong=1)
    gpu = api.Simulation(prob, mg)
    gpu.solver.set_solution_history(6)
    cpu = oracle.Simulation(prob, mg.n_levels, mg.nu_pre, mg.nu_post, mg.nu_coarse, mg.tol_mode,
                            mg.tol, mg.max_cycles, surface_prolong=1)
    gpu.start()
    cpu.start()
    for _ in range(100):
        gpu.step()
        cpu.step()
    g = gpu.state()
    c = cpu.state()
    k = slice(1, prob.nk + 1)
    assert g["it"] == c["it"] == 100
    assert g["vcycles"] < c["vcycles"]            # the guess saved cycles
    assert rel(g["t"], c["t"]) < 1e-12
    assert rel(g["Slip"][k], c["Slip"][k]) < 1e-8
    assert rel(g["psi"][k], c["psi"][k]) < 1e-8
    assert np.max(np.abs(g["V"][k] - c["V"][k]) / c["V"][k]) < 1e-10
    assert rel(g["Ts"][k] + prob.tau0[k], c["Ts"][k] + prob.tau0[k]) < 1e-10
    assert rel(g["U"], c["U"]) < 1e-10
    # the last solve is the step's refresh solve: its new slip carries the
    # last stage's slip rate (weight b_6 = 1/4), a direction no stored
    # solution's boundary contains, so its fit removes little; a fit is only
    # ever kept when it does not increase the misfit
    coef, misfit = gpu.solver.solution_history_fit()
    assert len(coef) == 5 and 0.0 <= misfit <= 1.0
    gpu.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_history_guess_saves_cycles_at_the_bench_tolerance(precision):
    cfg, prob = make_problem(129, mu_profile="layered", amb_perturb=0.05)
    # a fixed step, so both runs take the same steps: with adaptive steps at
    # this tolerance the step sequence follows the solves' round-off-level
    # differences and the two runs sample different times
    prob.ini_dt = prob.mindt = prob.maxdt = 3e5
    mg = config.MGConfig(n_levels=cfg.mg.n_levels, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1,
                         tol=1e-9, max_cycles=200, precision=precision, surface_prolong=1,
                         coarse_solve=1)
    out = {}
    for m in (0, 6):
        sim = api.Simulation(prob, mg)
        sim.solver.set_solution_history(m)
        sim.start()
        sim.step(40)
        out[m] = sim.state()
        sim.close()
    a, b = out[0], out[6]
    k = slice(1, prob.nk + 1)
    assert a["it"] == b["it"] == 40
    per_a = a["vcycles"] / a["solves"]
    per_b = b["vcycles"] / b["solves"]
    assert per_b < 0.8 * per_a, (per_a, per_b)
    # both runs solve to the same 1e-9 relative residual; their states agree
    # to what that tolerance lets through the RK error control
    assert b["t"] == a["t"]
    assert rel(b["Slip"][k], a["Slip"][k]) < 1e-7
    assert rel(b["psi"][k], a["psi"][k]) < 1e-7
    assert np.max(np.abs(b["V"][k] - a["V"][k]) / a["V"][k]) < 1e-6
    assert rel(b["U"], a["U"]) < 1e-7


def test_history_capacity_is_checked():
    cfg, prob = make_problem(33)
    sim = api.Simulation(prob, cfg.mg)
    with pytest.raises(_lib.QdError):
        sim.solver.set_solution_history(9)
    sim.solver.set_solution_history(8)
    sim.solver.set_solution_history(0)
    sim.close()
