"""GB300 kernels against the CPU oracle, through the C ABI.

Tolerances (FP64):
  * single smoother / V-cycle steps: 1e-12 relative to max|u| (the GPU uses
    fused multiply-adds and a precomputed 1/diag; the oracle rounds every
    operation as the reference's source reads);
  * converged solves, stress, slip rate: 1e-10 relative;
  * after 100 accepted RK43 steps: u, tau, V to 1e-10 and slip, psi to 1e-8
    relative (the drop-in's parity bar).
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


def oracle_medium(ni, nk, mu):
    return oracle.set_medium(ni, nk, mu)[1]


def make_problem(n=65, **kw):
    cfg = config.small(n, **kw)
    return cfg, problem.build_problem(cfg, homogenize=oracle_medium)


def random_U(prob, seed=0):
    rng = np.random.default_rng(seed)
    U = np.zeros((prob.nz, prob.nx))
    U[1:-1, 1:-1] = rng.normal(size=(prob.nk, prob.ni)) * 1e-3
    U[1:-1, 1] = rng.normal(size=prob.nk)          # fault column data
    U[1:-1, prob.ni] = rng.normal(size=prob.nk)    # remote column data
    return U


def compact(U):
    return np.ascontiguousarray(U[1:-1, 1:-1])


@pytest.fixture(scope="module", autouse=True)
def _libs(gpu_lib, oracle_lib):
    return gpu_lib


def test_set_medium_gpu_matches_oracle():
    cfg = config.small(65, mu_profile="layered", layer_depth_km=10.0)
    nx, nz = cfg.ni + 2, cfg.nk + 2
    mu_rows = problem.mu_profile(cfg, problem.depth_of_rows(cfg.nk, cfg.dh))
    mu = np.ascontiguousarray(np.repeat(mu_rows[:, None], nx, axis=1))
    want = oracle_medium(cfg.ni, cfg.nk, mu)
    got = api.set_medium(cfg.ni, cfg.nk, mu)
    assert rel(got, want) < 1e-13


@pytest.mark.parametrize("n", [33, 65])
def test_smoother_matches_oracle(n):
    cfg, prob = make_problem(n, mu_profile="layered", layer_depth_km=15.0)
    U = random_U(prob, 1)
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, cfg.mg)
    s.upload_u(U)
    s.smooth(3)
    got = compact(s.download_u())
    mg = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, cfg.mg.n_levels)
    u = compact(U).copy()
    f = np.zeros_like(u)
    for _ in range(3):
        mg.rbgs(u, f, 0, 0)
        mg.rbgs(u, f, 0, 1)
    assert rel(got, u) < 1e-12


@pytest.mark.parametrize("levels", [2, 4, 6])
def test_vcycle_matches_oracle(levels):
    cfg, prob = make_problem(129, mu_profile="layered", layer_depth_km=20.0)
    mg_cfg = config.MGConfig(n_levels=levels, nu_pre=2, nu_post=3, nu_coarse=7)
    U = random_U(prob, 2)
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, mg_cfg)
    s.upload_u(U)
    s.vcycle()
    s.vcycle()
    got = compact(s.download_u())
    mg = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, levels, 2, 3, 7)
    u = compact(U).copy()
    f = np.zeros_like(u)
    mg.vcycle(u, f)
    mg.vcycle(u, f)
    assert rel(got, u) < 1e-12
    r = np.zeros_like(u)
    mg.residual(r, u, f, 0)
    assert rel(s.residual_norm(), mg.norm2(r)) < 1e-9


@pytest.mark.parametrize("surface", [0, 1])
def test_vcycle_exact_coarse_solve_matches_oracle(surface):
    cfg, prob = make_problem(129, mu_profile="layered", layer_depth_km=20.0)
    mg_cfg = config.MGConfig(n_levels=5, nu_pre=2, nu_post=2, nu_coarse=0, surface_prolong=surface,
                             coarse_solve=1)
    U = random_U(prob, 7)
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, mg_cfg)
    s.upload_u(U)
    s.vcycle()
    s.vcycle()
    got = compact(s.download_u())
    mg = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, 5, 2, 2, 0, surface_prolong=surface,
                          coarse_solve=1)
    u = compact(U).copy()
    f = np.zeros_like(u)
    mg.vcycle(u, f)
    mg.vcycle(u, f)
    assert rel(got, u) < 1e-11


def test_mixed_solve_with_exact_coarse_solve():
    cfg, prob = make_problem(257, mu_profile="layered", layer_depth_km=8.0)
    base = dict(n_levels=6, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1, tol=1e-10, max_cycles=100,
                surface_prolong=1)
    U = random_U(prob, 8)
    res = {}
    for prec, cs in ((0, 0), (1, 1)):
        s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node,
                       config.MGConfig(**base, precision=prec, coarse_solve=cs))
        s.upload_u(U)
        cyc, rn, r0 = s.ode_solve()
        assert rn <= 1e-10 * r0
        res[(prec, cs)] = (cyc, compact(s.download_u()))
    assert res[(1, 1)][0] <= res[(0, 0)][0]
    assert rel(res[(1, 1)][1], res[(0, 0)][1]) < 1e-8


@pytest.mark.parametrize("precision", [0, 1])
def test_tail_sweeps_reach_the_same_solution(precision):
    """One pre- and one post-sweep on the coarse tail's levels (65 rows and
    below; qd_set_tail_sweeps) instead of V(2,2) there: the solve still
    meets 1e-10 of ||r0|| with at most one V-cycle more, and its u agrees
    with the default schedule's and with the oracle's solve to what that
    tolerance lets through."""
    cfg, prob = make_problem(257, mu_profile="layered", layer_depth_km=8.0)
    mg_cfg = config.MGConfig(n_levels=6, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1, tol=1e-10,
                             max_cycles=100, precision=precision, surface_prolong=1, coarse_solve=1)
    U = random_U(prob, 6)
    res = {}
    for tail in (0, 1):
        s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, mg_cfg)
        s.set_tail_sweeps(tail)
        s.upload_u(U)
        cyc, rn, r0 = s.ode_solve()
        assert rn <= 1e-10 * r0
        res[tail] = (cyc, compact(s.download_u()))
        if tail == 1:
            with pytest.raises(Exception):
                s.set_tail_sweeps(-1)
        s.close()
    assert res[1][0] <= res[0][0] + 1, (res[0][0], res[1][0])
    assert rel(res[1][1], res[0][1]) < 1e-8
    mg = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, 6, 2, 2, 32)
    u = compact(U).copy()
    mg.solve(u, tol_mode=1, tol=1e-12, max_cycles=200)
    assert rel(res[1][1], u) < 1e-8


def test_smoothing_pass_reaches_the_same_solution():
    """Mixed precision with the level-0 smoothing pass
    (qd_set_smooth_correction; ratio 1e6 alternates passes and V-cycles):
    solves from rough data meet 1e-10 of ||r0|| (the tolerance is checked
    after every correction), the smoothing passes are counted apart from the
    V-cycles, no two come in a row, and u agrees with the oracle's solution
    to what the tolerance lets through.  The FP64 solver refuses the pass."""
    cfg, prob = make_problem(257, mu_profile="layered", layer_depth_km=8.0)
    mg_cfg = config.MGConfig(n_levels=6, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1, tol=1e-10,
                             max_cycles=100, precision=1, surface_prolong=1, coarse_solve=1)
    mg = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, 6, 2, 2, 32)
    smooths = 0
    for seed in range(6):
        U = random_U(prob, 20 + seed)
        u = compact(U).copy()
        mg.solve(u, tol_mode=1, tol=1e-12, max_cycles=200)
        s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, mg_cfg)
        s.set_smooth_correction(1e6 if seed % 2 else 3.0)
        s.upload_u(U)
        cyc, rn, r0 = s.ode_solve()
        st = s.stats()
        assert rn <= 1e-10 * r0
        assert cyc == st["vcycles"] + st["smooth_corrections"]
        assert st["smooth_corrections"] <= st["vcycles"]
        smooths += st["smooth_corrections"]
        assert rel(compact(s.download_u()), u) < 1e-8
        with pytest.raises(Exception):
            s.set_smooth_correction(0.5)
        s.close()
    assert smooths > 0
    s64 = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node,
                     config.MGConfig(**{**mg_cfg.__dict__, "precision": 0}))
    with pytest.raises(Exception):
        s64.set_smooth_correction(2.5)
    s64.close()


def test_reference_schedule_solve_matches_oracle():
    """The reference's own schedule: 6 levels, V(32,32), absolute 1e-9."""
    cfg, prob = make_problem(129, mu_profile="layered", layer_depth_km=20.0)
    ref = config.reference_mg()
    ref.max_cycles = 1000
    U = random_U(prob, 3)
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, ref)
    Ug = U.copy()
    cyc, rn = s.ode_solve_host(Ug)
    mg = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, 6, 32, 32, 32)
    u = compact(U).copy()
    ocyc, orn, _ = mg.solve(u, tol_mode=0, tol=1e-9, max_cycles=1000)
    assert cyc == ocyc
    assert rn <= 1e-9 and orn <= 1e-9
    Uo = U.copy()
    Uo[1:-1, 1:-1] = u
    oracle.extend_crew(prob.ni, prob.nk, Uo)
    assert rel(Ug, Uo) < 1e-10


@pytest.mark.parametrize("precision", [0, 1])
def test_relative_tolerance_solve(precision):
    cfg, prob = make_problem(257, mu_profile="layered", layer_depth_km=8.0)
    mg_cfg = config.MGConfig(n_levels=6, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1, tol=1e-10,
                             max_cycles=100, precision=precision)
    U = random_U(prob, 4)
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, mg_cfg)
    s.upload_u(U)
    cyc, rn, r0 = s.ode_solve()
    assert rn <= 1e-10 * r0
    got = compact(s.download_u())
    mg = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, 6, 2, 2, 32)
    u = compact(U).copy()
    ocyc, orn, or0 = mg.solve(u, tol_mode=1, tol=1e-10, max_cycles=100)
    assert rel(r0, or0) < 1e-12
    if precision == 0:
        assert cyc == ocyc
    # both are within the tolerance of the exact discrete solution
    assert rel(got, u) < 1e-8


def test_fault_functions_match_oracle():
    cfg, prob = make_problem(65)
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, cfg.mg)
    s.fault_setup(prob)
    U = random_U(prob, 5) * 1e-2
    s.upload_u(U)
    Ts, Tn = s.eval_stress_on_fault()
    oTs, oTn = oracle.eval_stress_on_fault(prob.ni, prob.nk, prob.dh, U, prob.mu_node, prob.Tau_n0)
    k = slice(1, prob.nk + 1)
    assert rel(Ts[k], oTs[k]) < 1e-13
    assert np.array_equal(Tn[k], oTn[k])
    seed = np.zeros(prob.nz)
    V, it, rc = s.nrsearch(Ts, prob.psi, seed)
    assert rc == 0
    oV, oit, st = oracle.nrsearch(prob.nk, oTs, oTn, prob.a, prob.eta, prob.psi, prob.V0, seed,
                                  tau0=prob.tau0)
    assert st == 0
    assert np.max(np.abs(V[k] - oV[k]) / oV[k]) < 1e-10
    assert np.array_equal(it[k], oit[k])      # same iterate path from the reference's seed
    d = s.cal_dpsi(prob.psi, V)
    od = oracle.cal_dpsi(prob.nk, prob.psi, prob.b, oV, prob.f0, prob.V0, prob.L)
    assert rel(d[k], od[k]) < 1e-9


def test_newton_safeguard_recovers_where_reference_overflows():
    """fb/fa = 1200: the reference's first step overflows sinh (NaN, exit(0));
    the bracketed Newton returns the root."""
    cfg, prob = make_problem(33)
    p = prob
    p.a[:] = 0.005
    p.Tau_n0[:] = -10.0
    p.eta[:] = 4.0
    s = api.Solver(p.ni, p.nk, p.dh, p.mu_equi, p.mu_node, cfg.mg)
    s.fault_setup(p, with_tau0=False)
    Ts = np.full(p.nz, 60.0)
    psi = np.full(p.nz, 0.7)
    V, it, rc = s.nrsearch(Ts, psi, np.zeros(p.nz))
    assert rc == 0
    k = slice(1, p.nk + 1)
    x = np.arcsinh(V[k] / (2 * p.V0) * np.exp(psi[k] / p.a[k]))
    g = p.eta[k] * V[k] + p.a[k] * 10.0 * x - Ts[k]
    assert np.all(np.isfinite(V[k])) and np.max(np.abs(g)) < 1e-9 * 60.0


def test_newton_binary32_start_reaches_the_reference_root():
    """Newton start mode 1 (a binary32 solve of the log form, then the same
    FP64 iteration and stopping rule): over states from steady sliding to
    seismic slip rates, the slip rate equals the oracle's (the reference's
    iteration from x = 0) to 1e-12, in at most 3 FP64 steps where the
    reference's start takes up to 11; fb = 0 gives V = 0; the case where
    the reference's first step overflows is solved too."""
    cfg, prob = make_problem(65)
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, cfg.mg)
    s.fault_setup(prob)
    s.set_newton_start(1)
    k = slice(1, prob.nk + 1)
    rng = np.random.default_rng(9)
    for trial in range(4):
        psi = prob.psi.copy()
        psi[k] = rng.uniform(0.45, 0.85, prob.nk)
        fb = rng.uniform(-5.0, 40.0, prob.nz)
        fb[prob.nk // 2] = 0.0
        Ts = fb - prob.tau0
        seed = np.zeros(prob.nz)
        V, it, rc = s.nrsearch(Ts, psi, seed)
        assert rc == 0
        oV, oit, st = oracle.nrsearch(prob.nk, Ts, prob.Tau_n0, prob.a, prob.eta, psi, prob.V0, seed,
                                      tau0=prob.tau0)
        assert st == 0
        nz = oV[k] != 0.0
        assert np.max(np.abs(V[k][nz] - oV[k][nz]) / np.abs(oV[k][nz])) < 1e-12
        assert V[prob.nk // 2] == 0.0 and oV[prob.nk // 2] == 0.0
        assert it[k].max() <= 3 and oit[k].max() >= 7, (it[k].max(), oit[k].max())
    p = prob
    p.a[:] = 0.005
    p.Tau_n0[:] = -10.0
    p.eta[:] = 4.0
    s2 = api.Solver(p.ni, p.nk, p.dh, p.mu_equi, p.mu_node, cfg.mg)
    s2.fault_setup(p, with_tau0=False)
    s2.set_newton_start(1)
    Ts = np.full(p.nz, 60.0)
    psi = np.full(p.nz, 0.7)
    V, it, rc = s2.nrsearch(Ts, psi, np.zeros(p.nz))
    assert rc == 0
    x = np.arcsinh(V[k] / (2 * p.V0) * np.exp(psi[k] / p.a[k]))
    g = p.eta[k] * V[k] + p.a[k] * 10.0 * x - Ts[k]
    assert np.all(np.isfinite(V[k])) and np.max(np.abs(g)) < 1e-9 * 60.0
    with pytest.raises(Exception):
        s.set_newton_start(2)


def test_newton_binary32_start_keeps_the_rk_steps():
    """100 fixed RK43 steps (the 100-step bar's set-up) with Newton start
    mode 1 against the oracle (the reference's start) to the bar's
    tolerances, with fewer FP64 Newton steps than mode 0."""
    cfg, prob = make_problem(65)
    prob.ini_dt = prob.mindt = prob.maxdt = 3e5
    mg = config.MGConfig(n_levels=cfg.mg.n_levels, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1,
                         tol=1e-13, max_cycles=400, surface_prolong=1)
    cpu = oracle.Simulation(prob, mg.n_levels, mg.nu_pre, mg.nu_post, mg.nu_coarse, mg.tol_mode,
                            mg.tol, mg.max_cycles, surface_prolong=1)
    cpu.start()
    for _ in range(100):
        cpu.step()
    c = cpu.state()
    iters = []
    k = slice(1, prob.nk + 1)
    for mode in (0, 1):
        gpu = api.Simulation(prob, mg)
        gpu.solver.set_newton_start(mode)
        gpu.start()
        gpu.step(100)
        g = gpu.state()
        gpu.close()
        assert g["it"] == 100
        assert rel(g["t"], c["t"]) < 1e-12
        assert rel(g["Slip"][k], c["Slip"][k]) < 1e-8
        assert rel(g["psi"][k], c["psi"][k]) < 1e-8
        assert np.max(np.abs(g["V"][k] - c["V"][k]) / c["V"][k]) < 1e-10
        assert rel(g["U"], c["U"]) < 1e-10
        iters.append(g["newton_iters"])
    assert iters[1] < iters[0], iters


@pytest.mark.parametrize("surface", [0, 1])
def test_rk43_100_steps_match_oracle(surface):
    """100 accepted RK43 steps of the interseismic period, GPU vs oracle.

    Steady sliding at Vp in the velocity-weakening zone is an unstable
    equilibrium: perturbations grow like exp(t V/L), about 1e10 per decade
    here, so any two implementations that differ in the last bit diverge
    after a few simulated years, and round-off-level error estimates make
    the adaptive step sequence itself round-off driven.  Parity is therefore
    checked over one simulated year with the step fixed by the reference's
    own parameters (ini_dt = mindt = maxdt = 3e5 s; computeStepSize then
    always returns it), and solves tight enough (1e-13 relative) that the
    solver tolerance is not what differs.  Over this window an oracle run
    perturbed by 1e-14 in one node's prestress stays within 1e-13 of the
    unperturbed one."""
    cfg, prob = make_problem(65)
    prob.ini_dt = prob.mindt = prob.maxdt = 3e5
    mg = config.MGConfig(n_levels=cfg.mg.n_levels, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1,
                         tol=1e-13, max_cycles=400, surface_prolong=surface)
    gpu = api.Simulation(prob, mg)
    cpu = oracle.Simulation(prob, mg.n_levels, mg.nu_pre, mg.nu_post, mg.nu_coarse, mg.tol_mode,
                            mg.tol, mg.max_cycles, surface_prolong=surface)
    gpu.start()
    cpu.start()
    for _ in range(100):
        gpu.step()
        cpu.step()
    g = gpu.state()
    c = cpu.state()
    k = slice(1, prob.nk + 1)
    assert g["it"] == c["it"] == 100
    # the cycle count may differ by one where a residual norm sits at the
    # threshold; the states below are what must agree
    assert abs(g["vcycles"] - c["vcycles"]) <= 10
    assert rel(g["t"], c["t"]) < 1e-12 and rel(g["dt"], c["dt"]) < 1e-12
    assert rel(g["Slip"][k], c["Slip"][k]) < 1e-8
    assert rel(g["psi"][k], c["psi"][k]) < 1e-8
    assert np.max(np.abs(g["V"][k] - c["V"][k]) / c["V"][k]) < 1e-10
    assert rel(g["Ts"][k] + prob.tau0[k], c["Ts"][k] + prob.tau0[k]) < 1e-10   # total shear stress
    assert rel(g["U"], c["U"]) < 1e-10


def test_rk43_adaptive_steps_match_oracle():
    """The first adaptive steps (dt growing 5x per step from ini_dt, the
    accept/reject logic and the error estimate) against the oracle."""
    cfg, prob = make_problem(65)
    mg = config.MGConfig(n_levels=cfg.mg.n_levels, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1,
                         tol=1e-13, max_cycles=400, surface_prolong=1)
    gpu = api.Simulation(prob, mg)
    cpu = oracle.Simulation(prob, mg.n_levels, mg.nu_pre, mg.nu_post, mg.nu_coarse, mg.tol_mode,
                            mg.tol, mg.max_cycles, surface_prolong=1)
    gpu.start()
    cpu.start()
    for _ in range(6):
        gpu.step()
        cpu.step()
        g = gpu.state(with_u=False)
        c = cpu.state()
        assert rel(g["t"], c["t"]) < 1e-12 and rel(g["dt"], c["dt"]) < 1e-12
    k = slice(1, prob.nk + 1)
    assert np.max(np.abs(g["V"][k] - c["V"][k]) / c["V"][k]) < 1e-10
    assert rel(g["Slip"][k], c["Slip"][k]) < 1e-8


def test_host_buffer_step_equals_the_device_step():
    """qd_rk43_step_host (the state and the ghosted u on the host, uploaded,
    stepped, read back in one call) gives the same bits as qd_rk43_step on
    the device-resident state followed by the state and u read-backs, and
    its u carries extend_crew's ghost values."""
    cfg, prob = make_problem(65)
    outs = []
    for host in (False, True):
        sim = api.Simulation(prob, cfg.mg)
        sim.solver.set_solution_history(3)
        sim.start()
        sim.step(3)
        st = sim.solver.rk43_state()
        U = sim.solver.download_u()
        if host:
            for _ in range(4):
                assert sim.solver.rk43_step_host(1, st, U) == 1
        else:
            sim.step(4)
            st = sim.solver.rk43_state()
            U = sim.solver.download_u()
        outs.append((st, U))
        sim.close()
    (a, Ua), (b, Ub) = outs
    for key in ("Slip", "psi", "V", "dpsi", "Ts"):
        assert np.array_equal(a[key], b[key]), key
    assert a["t"] == b["t"] and a["dt"] == b["dt"] and a["it"] == b["it"]
    assert np.array_equal(Ua, Ub)
    Ue = Ub.copy()
    oracle.extend_crew(prob.ni, prob.nk, Ue)
    assert np.array_equal(Ue, Ub)


def test_gpu_runs_are_bitwise_reproducible():
    cfg, prob = make_problem(33)
    outs = []
    for _ in range(2):
        sim = api.Simulation(prob, cfg.mg)
        sim.start()
        sim.step(20)
        outs.append(sim.state())
        sim.close()
    for key in ("Slip", "psi", "V", "U"):
        assert np.array_equal(outs[0][key], outs[1][key]), key
    assert outs[0]["t"] == outs[1]["t"]


def test_f64_to_f32_rounding_matches_ieee():
    """The residual kernel's integer-pipe FP64 -> FP32 rounding (d2f_rne)
    equals IEEE round-to-nearest-even (numpy's cast) bit for bit: random
    values over the whole binary32 exponent range, exact ties with even and
    odd kept fractions, the overflow boundary, subnormal results, zeros,
    infinities and NaN."""
    import ctypes as C
    from qdeqcycle_fdm_gb300 import _lib
    rng = np.random.default_rng(7)
    x = [rng.uniform(-1, 1, 20000) * 10.0 ** rng.uniform(-46, 39, 20000)]
    # ties: fraction bits below the kept 23 are exactly one half
    frac = rng.integers(0, 1 << 23, 4000, dtype=np.uint64) << np.uint64(29)
    tie = frac | np.uint64(1 << 28)
    exp = rng.integers(1023 - 126, 1023 + 127, 4000).astype(np.uint64) << np.uint64(52)
    x.append((tie | exp).view(np.float64))
    x.append(((tie + np.uint64(1)) | exp).view(np.float64))   # just above a tie
    x.append(((tie - np.uint64(1)) | exp).view(np.float64))   # just below a tie
    fmax = float(np.finfo(np.float32).max)
    x.append(np.array([fmax, np.nextafter(fmax, np.inf), fmax * (1 + 2.0 ** -25), fmax * (1 + 2.0 ** -24),
                       2.0 ** -126, 2.0 ** -127, 2.0 ** -149, 2.0 ** -150, 2.0 ** -151, 1e-300,
                       0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 1.0 + 2.0 ** -24,
                       1.0 + 3 * 2.0 ** -24]))
    x = np.ascontiguousarray(np.concatenate(x))
    out = np.empty(x.size, dtype=np.float32)
    L = _lib.load()
    rc = L.qd_convert_f64_to_f32(x.ctypes.data_as(C.POINTER(C.c_double)),
                                 out.ctypes.data_as(C.POINTER(C.c_float)), x.size)
    assert rc == 0, L.qd_last_error().decode()
    with np.errstate(over="ignore"):
        ref = x.astype(np.float32)
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(out), nan)
    assert np.array_equal(out[~nan].view(np.uint32), ref[~nan].view(np.uint32))


def test_double_float_split_matches_its_definition():
    """The mixed residual's split x = hi + lo (d_split), on the integer and
    FP32 pipes: hi is x truncated to binary32's 24 significant bits, lo the
    remainder rounded to nearest binary32, bit for bit against the same on
    the host, so |hi + lo - x| <= 2^-48 |x|; |x| < 2^-74 and zeros give
    (+-0, 0), |x| >= 2^128 +-inf, NaN stays NaN."""
    import ctypes as C
    from qdeqcycle_fdm_gb300 import _lib
    rng = np.random.default_rng(11)
    x = rng.uniform(-1, 1, 40000) * 10.0 ** rng.uniform(-30, 38, 40000)
    x = np.concatenate([x, [0.0, -0.0, 1.0, -1.0, 2.0 ** -74, -(2.0 ** -74), np.nextafter(2.0 ** -74, 0),
                            1e-40, 1e39, -1e39, np.inf, -np.inf, np.nan, 1.0 + 2.0 ** -52, 3.0 - 2.0 ** -51,
                            np.nextafter(2.0 ** 128, 0), 2.0 ** 128]])
    x = np.ascontiguousarray(x)
    hi = np.empty(x.size, dtype=np.float32)
    lo = np.empty(x.size, dtype=np.float32)
    L = _lib.load()
    fp = C.POINTER(C.c_float)
    rc = L.qd_split_f64(x.ctypes.data_as(C.POINTER(C.c_double)), hi.ctypes.data_as(fp), lo.ctypes.data_as(fp),
                        x.size)
    assert rc == 0, L.qd_last_error().decode()
    low29 = np.uint64((1 << 29) - 1)
    with np.errstate(over="ignore", invalid="ignore"):
        ok = np.isfinite(x) & (np.abs(x) >= 2.0 ** -74) & (np.abs(x) < 2.0 ** 128)
        hi_ref = (x.view(np.uint64) & ~low29).view(np.float64)
        lo_ref = np.where(ok, x - hi_ref, 0.0).astype(np.float32)
        assert np.array_equal(hi[ok].view(np.uint32), hi_ref[ok].astype(np.float32).view(np.uint32))
        assert np.array_equal(lo[ok], lo_ref[ok])      # by value: a zero lo may carry x's sign
        err = np.abs(hi[ok].astype(np.float64) + lo[ok].astype(np.float64) - x[ok])
        assert np.all(err <= 2.0 ** -48 * np.abs(x[ok]))
    tiny = np.abs(x) < 2.0 ** -74
    assert np.all(hi[tiny] == 0.0) and np.all(lo[tiny] == 0.0)
    assert np.array_equal(np.signbit(hi[tiny]), np.signbit(x[tiny]))
    over = np.isinf(x) | (np.isfinite(x) & (np.abs(x) >= 2.0 ** 128))
    assert np.all(np.isinf(hi[over])) and np.array_equal(np.sign(hi[over]), np.sign(x[over]))
    assert np.all(lo[over] == 0.0)
    assert np.isnan(hi[np.isnan(x)]).all() and np.all(lo[np.isnan(x)] == 0.0)


def test_mixed_residual_matches_fp64_residual():
    """The mixed solver's level-0 residual, evaluated in double-float
    arithmetic on the FP32 and integer pipes, reports the norm that the
    oracle's FP64 residual of the same u gives to 1e-4 (measured: 4e-6):
    after a solve to 1e-10 of ||r0|| (random boundary data, the finest
    tolerance the tests use) and after one to 1e-3."""
    cfg, prob = make_problem(257, mu_profile="layered", layer_depth_km=8.0)
    mg = oracle.Multigrid(prob.ni, prob.nk, prob.dh, prob.mu_equi, 6, 2, 2, 32)
    U = random_U(prob, 5)
    for tol in (1e-10, 1e-3):
        s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node,
                       config.MGConfig(n_levels=6, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1, tol=tol,
                                       max_cycles=100, precision=1, surface_prolong=1, coarse_solve=1))
        s.upload_u(U)
        cyc, rn, r0 = s.ode_solve()
        got = compact(s.download_u()).copy()
        s.close()
        r = np.zeros_like(got)
        mg.residual(r, got, np.zeros_like(got), 0)
        rn64 = mg.norm2(r)
        assert abs(rn - rn64) <= 1e-4 * rn64, (tol, rn, rn64)
        assert rn <= tol * r0
