"""Failure paths of the stepping loop, each made on the host, none of them
faulting or hanging the GPU.

The reference stops the process on a NaN in the Newton solve for slip rate
(fault.cpp:211-225), retries an attempt at most 100 times
(odeSolver.cpp:1466-1472) and loops on the multigrid with no cap
(odeSolver.cpp:696).  Here every one of those ends in a status code the
caller reads, and the solver stays usable:
  * a NaN in psi or an infinity in the slip (the boundary data), written
    into the state from the host, ends qd_rk43_step with QD_ERR_NEWTON or
    QD_ERR_NOT_CONVERGED at the attempt that met it;
  * a tolerance out of reach stops the device-driven solve loop at its cap
    (max_cycles, or QD_SOLVE_GRAPH_MAX_CYCLES when uncapped);
  * a staging wait that nothing completes gives up after its poll limit
    and the call reports it (qd_probe_bounded_wait).
"""
import numpy as np
import pytest

import oracle
from qdeqcycle_fdm_gb300 import _lib, api, config, problem
from qdeqcycle_fdm_gb300._lib import QdError

pytestmark = pytest.mark.gpu

GRAPH_CAP = 10000     # QD_SOLVE_GRAPH_MAX_CYCLES in include/qdeq.h


def _prob(n=33, **kw):
    cfg = config.small(n, **kw)
    return cfg, problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])


def _started(mg=None, precision=0):
    cfg, prob = _prob()
    mg = mg or config.MGConfig(**{**cfg.mg.__dict__, "precision": precision})
    sim = api.Simulation(prob, mg)
    sim.start()
    sim.step(2)
    return prob, sim


@pytest.mark.parametrize("precision", [0, 1])
def test_nan_in_psi_ends_the_step_with_a_newton_status(gpu_lib, precision):
    prob, sim = _started(precision=precision)
    st = sim.solver.rk43_state()
    psi = st["psi"].copy()
    psi[prob.nk // 2] = np.nan
    sim.solver.rk43_set_state(st["Slip"], psi, st["V"], st["dpsi"], st["t"], st["dt"], st["errA"][0],
                              st["errA"][1], st["it"])
    a0 = sim.solver.stats()["attempts"]
    with pytest.raises(QdError) as e:
        sim.step(1)
    assert e.value.code == _lib.QD_ERR_NEWTON, str(e.value)
    assert "Newton" in str(e.value)
    # the step ended at the attempt that met the NaN, not after 100 retries
    assert sim.solver.stats()["attempts"] - a0 == 1
    # the oracle reports the same failure as a status (the reference exits)
    cfg, _ = _prob()
    cpu = oracle.Simulation(prob, cfg.mg.n_levels, cfg.mg.nu_pre, cfg.mg.nu_post, cfg.mg.nu_coarse,
                            cfg.mg.tol_mode, cfg.mg.tol, cfg.mg.max_cycles)
    cpu.start()
    ck = {"Slip": st["Slip"], "psi": psi, "t": st["t"], "dt": st["dt"], "errA0": st["errA"][0],
          "errA1": st["errA"][1], "it": st["it"]}
    assert cpu.resume(ck) != 0
    # the solver is usable again after a fresh start
    sim.start()
    assert sim.step(2) == 2
    sim.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_infinite_slip_ends_the_step_with_a_status(gpu_lib, precision):
    prob, sim = _started(precision=precision)
    st = sim.solver.rk43_state()
    slip = st["Slip"].copy()
    slip[3] = np.inf
    sim.solver.rk43_set_state(slip, st["psi"], st["V"], st["dpsi"], st["t"], st["dt"], st["errA"][0],
                              st["errA"][1], st["it"])
    with pytest.raises(QdError) as e:
        sim.step(1)
    assert e.value.code in (_lib.QD_ERR_NOT_CONVERGED, _lib.QD_ERR_NEWTON), str(e.value)
    sim.start()
    assert sim.step(1) == 1
    sim.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_unreachable_tolerance_stops_at_the_cycle_cap(gpu_lib, precision):
    cfg, prob = _prob()
    # an absolute tolerance far below the round-off floor of the residual,
    # with rough boundary data: a solution linear in x (constant data on a
    # medium layered in depth) is one the mixed residual's double-float
    # arithmetic resolves exactly, its residual rounding to zero
    rng = np.random.default_rng(3)
    for cap, want in ((7, 7), (0, GRAPH_CAP)):
        mg = config.MGConfig(**{**cfg.mg.__dict__, "tol_mode": 0, "tol": 1e-300, "max_cycles": cap,
                                "precision": precision})
        s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, mg)
        U = prob.U.copy()
        U[1:-1, 1] = rng.normal(size=prob.nk)          # fault column
        U[1:-1, prob.ni] = rng.normal(size=prob.nk)    # remote column
        s.upload_u(U)
        with pytest.raises(QdError) as e:
            s.ode_solve()
        assert e.value.code == _lib.QD_ERR_NOT_CONVERGED
        assert s.stats()["vcycles"] == want, (cap, s.stats()["vcycles"])
        s.close()


def test_bounded_staging_wait_gives_up_and_is_reported(gpu_lib):
    prob, sim = _started(precision=1)
    rc, msg = sim.solver.probe_bounded_wait(1000)
    assert rc == _lib.QD_ERR_CUDA
    assert "staging" in msg
    # the status stays set for the run ...
    with pytest.raises(QdError):
        sim.step(1)
    # ... and a new run clears it: the context is intact
    sim.start()
    assert sim.step(2) == 2
    assert sim.solver.probe_bounded_wait(0)[0] == _lib.QD_ERR_ARG
    sim.close()
