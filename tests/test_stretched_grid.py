"""The grid stretched in depth (config 2): the metric form of the operator.

The reference's grid is uniform (coord.cpp:18,27); a stretched grid is this
project's own discretisation, so the oracle is the only reference: the CPU oracle
applies the metric J = dz/dzeta as x-face moduli mu J and z-face moduli
mu / J on the uniform computational grid.  Here:
  * with J = 1 the metric code path reproduces the uniform oracle bit for bit;
  * the metric discretisation converges at second order to a harmonic
    function that meets the problem's boundary conditions
    (u = cos(pi z / D) sinh(pi (L - x) / D): Dirichlet columns, mirrored rows);
  * the mapping puts 4x finer rows over the fault zone;
  * on the GPU, the mapped coefficients give V-cycles, solves and RK43 steps
    that match the oracle's.
"""
import numpy as np
import pytest

import oracle
from qdeqcycle_fdm_gb300 import api, config, problem


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def _stretched(n, **kw):
    cfg = config.config2().replace(ni=n, nk=n, name=f"config2_{n}", **kw)
    lv = int(round(np.log2(n - 1))) - 2
    cfg.mg = config.MGConfig(n_levels=lv, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1, tol=1e-10,
                             max_cycles=200, precision=0, surface_prolong=1, coarse_solve=1)
    return cfg, problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])


def test_mapping_refines_the_fault_zone():
    cfg = config.config2()
    depth, jrow = problem.depth_metric(cfg)
    assert depth.shape == (cfg.nk + 2,) and jrow.shape == (2 * (cfg.nk + 2) - 1,)
    d = depth[1:-1]
    assert abs(d[0] - 40e3) < 1e-6 and abs(d[-1]) < 1e-9         # compact row 0 deepest, last at the surface
    dz = -np.diff(d)
    fine, coarse = dz[d[1:] < 18e3], dz[d[:-1] > 30e3]
    assert np.allclose(fine, fine[-1], rtol=1e-6) and np.allclose(coarse, coarse[0], rtol=1e-6)
    assert abs(coarse[0] / fine[-1] - 4.0) < 1e-5
    # the cohesive zone with Dc = 2 mm spans at least 8 rows of the fine zone
    lam = 0.6 * cfg.mu_gpa * 1e9 * cfg.Dc_m / (cfg.b * cfg.sigma_n_mpa * 1e6)
    assert lam / fine[-1] >= 8.0
    # J at the faces is the row spacing over the computational spacing
    dh = cfg.dh
    faces = jrow[3:2 * cfg.nk:2]                   # staggered rows between compact rows j, j+1
    assert np.max(np.abs(faces - dz / dh) / faces) < 2e-3


def test_unit_metric_reproduces_the_uniform_oracle(oracle_lib):
    cfg = config.small(65, mu_profile="layered", layer_depth_km=20.0)
    prob = problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])
    rng = np.random.default_rng(3)
    u0 = rng.normal(size=(prob.nk, prob.ni))
    ones = np.ones(2 * prob.nz - 1)
    outs = []
    for jr in (None, ones):
        m = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, 4, 2, 2, 8, jrow=jr)
        u = u0.copy()
        f = np.zeros_like(u)
        m.vcycle(u, f)
        outs.append(u)
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("ratio", [1.0, 4.0])
def test_metric_operator_converges_at_second_order(oracle_lib, ratio):
    errs = []
    for n in (65, 129, 257):
        cfg = config.config2().replace(ni=n, nk=n, stretch_ratio=ratio, stretch_width=0.05)
        depth, jrow = problem.depth_metric(cfg)
        D = cfg.domain_m
        x = np.arange(n) * cfg.dh
        z = depth[1:-1]
        exact = np.cos(np.pi * z / D)[:, None] * np.sinh(np.pi * (D - x) / D)[None, :]
        mu = np.full((n + 2, n + 2), 30.0)
        me = oracle.set_medium(n, n, mu)[1]
        lv = int(round(np.log2(n - 1))) - 2
        m = oracle.Multigrid(n, n, cfg.dh, me, lv, 2, 2, 32, surface_prolong=1, coarse_solve=1, jrow=jrow)
        u = np.zeros((n, n))
        u[:, 0] = exact[:, 0]
        u[:, -1] = exact[:, -1]
        cyc, rn, r0 = m.solve(u, tol_mode=1, tol=1e-13, max_cycles=200)
        assert rn <= 1e-13 * r0
        errs.append(np.max(np.abs(u - exact)) / np.max(np.abs(exact)))
    rates = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(rates) > 1.8, (errs, rates)


@pytest.mark.gpu
def test_gpu_vcycle_on_stretched_grid_matches_oracle(gpu_lib, oracle_lib):
    cfg, prob = _stretched(257, mu_profile="layered", layer_depth_km=6.0)
    rng = np.random.default_rng(4)
    U = np.zeros((prob.nz, prob.nx))
    U[1:-1, 1:-1] = rng.normal(size=(prob.nk, prob.ni)) * 1e-3
    U[1:-1, 1] = rng.normal(size=prob.nk)
    U[1:-1, prob.ni] = rng.normal(size=prob.nk)
    for surface, exact in ((0, 0), (1, 1)):
        mg = config.MGConfig(n_levels=6, nu_pre=2, nu_post=2, nu_coarse=8, surface_prolong=surface,
                             coarse_solve=exact)
        s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, mg, jrow=prob.jrow)
        s.upload_u(U)
        s.vcycle()
        got = s.download_u()[1:-1, 1:-1]
        m = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, 6, 2, 2, 8, surface_prolong=surface,
                             coarse_solve=exact, jrow=prob.jrow)
        u = np.ascontiguousarray(U[1:-1, 1:-1])
        f = np.zeros_like(u)
        m.vcycle(u, f)
        assert rel(got, u) < 1e-12, (surface, exact)
        s.close()


@pytest.mark.gpu
def test_gpu_mixed_solve_on_stretched_grid_matches_oracle(gpu_lib, oracle_lib):
    cfg, prob = _stretched(513)
    rng = np.random.default_rng(5)
    U = np.zeros((prob.nz, prob.nx))
    U[1:-1, 1] = rng.normal(size=prob.nk)
    U[1:-1, prob.ni] = rng.normal(size=prob.nk)
    mg = config.MGConfig(**{**cfg.mg.__dict__, "precision": 1, "tol": 1e-9})
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, mg, jrow=prob.jrow)
    s.upload_u(U)
    cyc, rn, r0 = s.ode_solve()
    assert rn <= 1e-9 * r0
    got = s.download_u()[1:-1, 1:-1]
    m = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, cfg.mg.n_levels, 2, 2, 32, surface_prolong=1,
                         coarse_solve=1, jrow=prob.jrow)
    u = np.ascontiguousarray(U[1:-1, 1:-1])
    ocyc, orn, or0 = m.solve(u, tol_mode=1, tol=1e-13, max_cycles=200)
    assert rel(r0, or0) < 1e-12
    assert rel(got, u) < 1e-8
    s.close()


@pytest.mark.gpu
def test_gpu_rk43_on_stretched_grid_matches_oracle(gpu_lib, oracle_lib):
    """30 fixed steps (dt 3e5 s) from steady sliding on a 129^2 stretched
    grid with config 2's friction: the FP64 drop-in against the oracle to
    the 100-step bar's tolerances (solves to 1e-13)."""
    cfg, prob = _stretched(129)
    prob.ini_dt = prob.mindt = prob.maxdt = 3e5
    mg = config.MGConfig(**{**cfg.mg.__dict__, "tol": 1e-13, "max_cycles": 400})
    gpu = api.Simulation(prob, mg)
    cpu = oracle.Simulation(prob, mg.n_levels, 2, 2, 32, 1, 1e-13, 400, surface_prolong=1, coarse_solve=1)
    gpu.start()
    cpu.start()
    for _ in range(30):
        gpu.step()
        cpu.step()
    g, c = gpu.state(), cpu.state()
    k = slice(1, prob.nk + 1)
    assert g["it"] == c["it"] == 30
    assert rel(g["Slip"][k], c["Slip"][k]) < 1e-8
    assert rel(g["psi"][k], c["psi"][k]) < 1e-8
    assert np.max(np.abs(g["V"][k] - c["V"][k]) / c["V"][k]) < 1e-10
    assert rel(g["U"], c["U"]) < 1e-10
    gpu.close()
