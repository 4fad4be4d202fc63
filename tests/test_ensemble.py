"""Batched ensemble (qd_ensemble_step): several instances of different grids
and parameters advanced together follow exactly the runs each would make on
its own, and the instance generator draws config 4's parameter ranges."""
import numpy as np
import pytest

from qdeqcycle_fdm_gb300 import config


def test_ensemble_instances_follow_the_config_ranges():
    for i in range(20):
        c = config.ensemble_instance(257, i)
        assert 0.002 <= c.b - c.a_shallow <= 0.006
        assert 2e-3 <= c.Dc_m <= 20e-3 and 20 <= c.sigma_n_mpa <= 80
        assert 10 <= c.seis_depth_km <= 16 and 25 <= c.mu_gpa <= 35
        assert c.mg.n_levels == 7
    assert config.ensemble_instance(257, 3) == config.ensemble_instance(257, 3)
    assert config.ensemble_instance(1025, 0).mg.n_levels == 9


@pytest.mark.gpu
def test_ensemble_step_matches_separate_runs():
    from qdeqcycle_fdm_gb300 import api, problem
    cfgs = [config.ensemble_instance(n, i) for i, n in enumerate((33, 65, 33))]
    probs = [problem.build_problem(c) for c in cfgs]

    def run(together):
        sims = [api.Simulation(p, c.mg) for p, c in zip(probs, cfgs)]
        for s in sims:
            s.start()
        if together:
            done = api.ensemble_step(sims, 12)
        else:
            done = [s.step(12) for s in sims]
        out = [s.state() for s in sims]
        for s in sims:
            s.close()
        return done, out

    d1, a = run(True)
    d2, b = run(False)
    assert d1 == d2 == [12, 12, 12]
    for x, y in zip(a, b):
        for k in ("Slip", "psi", "V", "U"):
            assert np.array_equal(x[k], y[k]), k
        assert x["t"] == y["t"] and x["vcycles"] == y["vcycles"]
