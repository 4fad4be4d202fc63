"""Restart from a fault-state checkpoint (Slip, psi, t, dt, the error
history and the step count): the oracle and the GPU each continue bit for
bit from their own checkpoint given the solved u, the GPU matches the oracle
after a restart from the zero-interior guess, and the committed mid-cycle
checkpoints of config 1 load with the sizes they claim."""
import numpy as np
import pytest

import oracle
from qdeqcycle_fdm_gb300 import api, checkpoints, config, problem

K = slice(1, 34)


def _prob(n=33):
    cfg = config.small(n, mu_profile="layered", amb_perturb=0.05)
    return cfg, problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])


def _oracle(prob, mg):
    return oracle.Simulation(prob, mg.n_levels, mg.nu_pre, mg.nu_post, mg.nu_coarse, mg.tol_mode, mg.tol,
                             mg.max_cycles)


def test_oracle_resume_continues_bit_for_bit(oracle_lib):
    cfg, prob = _prob()
    a = _oracle(prob, cfg.mg)
    a.start()
    for _ in range(12):
        a.step()
    mid = a.state()
    for _ in range(8):
        a.step()
    want = a.state()
    b = _oracle(prob, cfg.mg)
    assert b.resume(checkpoints.from_state(mid), U=mid["U"]) == 0
    for _ in range(8):
        b.step()
    got = b.state()
    for key in ("Slip", "psi", "V", "U"):
        assert np.array_equal(got[key], want[key]), key
    assert got["t"] == want["t"] and got["dt"] == want["dt"] and got["it"] == want["it"] == 20


def test_checkpoint_file_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    st = {"Slip": rng.normal(size=35), "psi": rng.normal(size=35), "t": 1.5e9, "dt": 0.0164,
          "errA0": 3e-8, "errA1": 5e-8, "it": 6077}
    f = str(tmp_path / "ck.npz")
    checkpoints.save(f, st, {"name": "x"})
    got = checkpoints.load(f)
    for k in checkpoints.KEYS:
        assert np.array_equal(got[k], st[k]), k
    assert got["meta"] == {"name": "x"}


@pytest.mark.parametrize("name", ["config1_1025_rupture3", "config1_1025_interseismic3"])
def test_committed_checkpoints_load(name):
    ck = checkpoints.load(name)
    assert ck["Slip"].shape == (1027,) and ck["psi"].shape == (1027,)
    assert ck["meta"]["config"] == "config1_1025" and ck["meta"]["name"] == name
    assert ck["t"] > 0 and ck["dt"] > 0 and ck["it"] > 0
    assert np.all(np.isfinite(ck["Slip"][1:-1])) and np.all(np.isfinite(ck["psi"][1:-1]))


@pytest.mark.gpu
def test_gpu_resume_continues_bit_for_bit(gpu_lib):
    cfg, prob = _prob()
    a = api.Simulation(prob, cfg.mg)
    a.start()
    a.step(12)
    mid = a.state()
    a.step(8)
    want = a.state()
    b = api.Simulation(prob, cfg.mg)
    b.resume(checkpoints.from_state(mid), U=mid["U"])
    b.step(8)
    got = b.state()
    for key in ("Slip", "psi", "V", "U"):
        assert np.array_equal(got[key], want[key]), key
    assert got["t"] == want["t"] and got["dt"] == want["dt"]
    a.close()
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_resume_matches_oracle(gpu_lib, oracle_lib, precision):
    """Both restart from the oracle's checkpoint after 15 steps with the
    zero-interior guess, then take 10 steps of the checkpoint's dt (fixed:
    near steady sliding the error estimate sits at round-off and the
    adaptive step sequence would be round-off driven)."""
    cfg, prob = _prob()
    c = _oracle(prob, cfg.mg)
    c.start()
    for _ in range(15):
        c.step()
    ck = checkpoints.from_state(c.state())
    dt = ck["dt"]
    params = (prob.tmax, dt, dt, dt, prob.totTol, 2**31 - 1)
    cpu = _oracle(prob, cfg.mg)
    cpu.set_params(*params)
    assert cpu.resume(ck) == 0
    mg = config.MGConfig(**{**cfg.mg.__dict__, "precision": precision})
    gpu = api.Simulation(prob, mg)
    gpu.resume(ck, params=params)
    for _ in range(10):
        cpu.step()
    gpu.step(10)
    g, o = gpu.state(), cpu.state()
    assert g["it"] == o["it"] == ck["it"] + 10
    assert abs(g["t"] - o["t"]) <= 1e-15 * o["t"]
    vtol = 1e-10 if precision == 0 else 1e-7
    assert np.max(np.abs(g["V"][K] - o["V"][K]) / o["V"][K]) < vtol
    assert np.max(np.abs(g["Slip"][K] - o["Slip"][K])) < 1e-8 * np.max(np.abs(o["Slip"][K]))
    gpu.close()
