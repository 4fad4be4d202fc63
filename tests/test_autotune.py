"""The autotuner (qd_autotune) and the tile box widths it chooses between.

  * every box width the tuner may pick leaves the FP64 V-cycle exact: two
    V-cycles match the oracle to 1e-12, as with the default tiles;
  * tuning leaves the simulation as it found it (u bit for bit, the solve
    counters), keeps a setting at least as fast as the one it started from,
    and the run continues with it; with a solution history it times the
    replayed last solve, which starts one V-cycle or so from the tolerance.
"""
import numpy as np
import pytest

import oracle
from qdeqcycle_fdm_gb300 import api, config, problem

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module", autouse=True)
def _libs(gpu_lib, oracle_lib):
    return gpu_lib


@pytest.mark.parametrize("boxes", [(96, 96), (128, 128), (128, 64), (64, 128)])
def test_tile_widths_keep_the_vcycle_exact(boxes):
    cfg = config.small(257, mu_profile="layered", layer_depth_km=20.0)
    prob = problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])
    mg_cfg = config.MGConfig(n_levels=4, nu_pre=2, nu_post=3, nu_coarse=7)
    rng = np.random.default_rng(5)
    U = np.zeros((prob.nz, prob.nx))
    U[1:-1, 1:-1] = rng.normal(size=(prob.nk, prob.ni)) * 1e-3
    U[1:-1, 1] = rng.normal(size=prob.nk)
    U[1:-1, prob.ni] = rng.normal(size=prob.nk)
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, mg_cfg)
    s.set_tiles(*boxes)
    s.upload_u(U)
    s.vcycle()
    s.vcycle()
    got = np.ascontiguousarray(s.download_u()[1:-1, 1:-1])
    s.close()
    mg = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, 4, 2, 3, 7)
    u = np.ascontiguousarray(U[1:-1, 1:-1]).copy()
    f = np.zeros_like(u)
    mg.vcycle(u, f)
    mg.vcycle(u, f)
    assert rel(got, u) < 1e-12


def test_autotune_restores_the_state_and_keeps_the_faster_setting():
    cfg = config.small(257, mu_profile="layered", amb_perturb=0.05)
    prob = problem.build_problem(cfg)
    import dataclasses
    mg = dataclasses.replace(cfg.mg, precision=1, surface_prolong=1, coarse_solve=1, tol=1e-9)
    sim = api.Simulation(prob, mg)
    sim.start()
    sim.step(5)
    before = sim.state()
    t = sim.solver.autotune(2)
    after = sim.state()
    assert np.array_equal(before["U"], after["U"])
    for k in ("solves", "vcycles", "steps", "attempts"):
        assert before[k] == after[k], k
    assert t["candidates"] >= 2
    assert t["us_best"] <= t["us_initial"]
    assert (t["nu_pre"], t["nu_post"]) in {(1, 1), (2, 2), (3, 3), (4, 4), (1, 2), (2, 1), (2, 3), (3, 2)}
    assert t["box_up"] in (64, 96, 128) and t["box_down"] in (64, 96, 128)
    assert t["cycles_best"] >= 1 and t["replayed"] == 0
    sim.step(5)                      # the run goes on with the tuned setting
    assert sim.state(with_u=False)["steps"] == 10
    sim.close()


def test_autotune_replays_the_history_solve():
    cfg = config.small(257, mu_profile="layered", amb_perturb=0.05)
    prob = problem.build_problem(cfg)
    import dataclasses
    mg = dataclasses.replace(cfg.mg, precision=1, surface_prolong=1, coarse_solve=1, tol=1e-9)
    sim = api.Simulation(prob, mg)
    sim.solver.set_solution_history(4)
    sim.start()
    sim.step(5)
    # a tolerance the replayed solve does not start within, so that it takes
    # cycles (a replay that takes none ranks nothing and is not used)
    sim.solver.set_options(dataclasses.replace(mg, tol=1e-12))
    before = sim.state()
    t = sim.solver.autotune(2)
    after = sim.state()
    assert t["replayed"] == 1
    assert np.array_equal(before["U"], after["U"])
    for k in ("solves", "vcycles", "steps", "attempts"):
        assert before[k] == after[k], k
    # the replayed solve starts from a history guess: a few cycles, against
    # the many of a solve from a zero interior
    assert 1 <= t["cycles_best"] <= 5 and t["us_best"] <= t["us_initial"]
    sim.step(5)
    assert sim.state(with_u=False)["steps"] == 10
    sim.close()
