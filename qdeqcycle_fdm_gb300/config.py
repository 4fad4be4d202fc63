"""Named workloads of the quasi-dynamic antiplane earthquake-cycle path.

Each config fixes the grid, the elastic medium, the rate-and-state friction,
the time-integration tolerances and the multigrid schedule.  Parameters the
reference hard-codes live in ``SetParams.cpp:3-30`` (time stepping and grid),
``fault.cpp:85-120`` (friction) and ``odeSolver.cpp:2-4,297-305`` (multigrid,
medium); here they are data.

Simulated years are 365.25-day years.  (The reference's ``tmax`` counts
360-day years, ``SetParams.cpp:11-12``.)
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field

YEAR_S = 365.25 * 86400.0


@dataclass
class MGConfig:
    n_levels: int = 6          # odeSolver.cpp:3
    nu_pre: int = 32           # odeSolver.cpp:4 (n_cycles: smooth() repeats)
    nu_post: int = 32
    nu_coarse: int = 32
    tol_mode: int = 0          # 0: absolute ||r||2 (odeSolver.cpp:689); 1: relative
    tol: float = 1e-9
    max_cycles: int = 0        # 0 = uncapped, as the reference
    precision: int = 0         # 0: FP64; 1: FP32 V-cycles inside FP64 refinement
    surface_prolong: int = 0   # 1: coarse correction also on the free-surface row
    coarse_solve: int = 0      # 1: exact (dense) solve on the coarsest level


@dataclass
class ProblemConfig:
    name: str
    ni: int                    # nodes off-fault (x), GRID.ni
    nk: int                    # nodes along the fault (depth), GRID.nk
    domain_m: float = 40e3     # square domain edge
    mu_profile: str = "uniform"    # "uniform" | "layered"
    mu_gpa: float = 30.0
    mu_surface_gpa: float = 20.0   # layered: linear from the surface ...
    mu_deep_gpa: float = 32.0      # ... to this value at layer_depth_km
    layer_depth_km: float = 4.0
    cs_kms: float = 3.3
    # rate-and-state (aging law); a(z): a_shallow to seis_depth, linear to a_deep
    a_shallow: float = 0.008
    a_deep: float = 0.024
    seis_depth_km: float = 12.0
    taper_depth_km: float = 16.0
    b: float = 0.012
    Dc_m: float = 0.006
    sigma_n_mpa: float = 40.0
    f0: float = 0.6
    V0: float = 1e-6
    Vp: float = 1e-9
    amb_perturb: float = 0.0   # uniform +-fraction perturbation of a-b per node
    # depth stretching (1: the reference's uniform grid): the row spacing is
    # stretch_ratio times larger below a tanh transition centred at
    # stretch_depth_km, of width stretch_width in the normalised depth
    # coordinate (see problem.depth_metric)
    stretch_ratio: float = 1.0
    stretch_depth_km: float = 21.0
    stretch_width: float = 0.01
    seed: int = 12345
    prestress: bool = True     # tau0 so that V = Vp at t = 0 with u = 0
    # time stepping (SetParams.cpp:14-17)
    years: float = 300.0
    ini_dt: float = 1e-3
    mindt: float = 1e-5
    maxdt: float = 1e8
    totTol: float = 1e-7
    maxNumSteps: int = 100000000
    mg: MGConfig = field(default_factory=MGConfig)

    @property
    def dh(self) -> float:
        return self.domain_m / (self.nk - 1)

    def replace(self, **kw) -> "ProblemConfig":
        return dataclasses.replace(self, **kw)


def reference_mg() -> MGConfig:
    """The reference's multigrid: 6 levels, V(32,32), absolute 1e-9."""
    return MGConfig(6, 32, 32, 32, 0, 1e-9, 0, 0)


def config0() -> ProblemConfig:
    """129x129 FP64, uniform mu = 30 GPa, 5-level V(2,2) to 1e-10 relative."""
    return ProblemConfig(name="config0_129", ni=129, nk=129, mu_profile="uniform",
                         years=300.0,
                         mg=MGConfig(n_levels=5, nu_pre=2, nu_post=2, nu_coarse=32,
                                     tol_mode=1, tol=1e-10, max_cycles=200))


def config1() -> ProblemConfig:
    """1025x1025 FP64, layered mu 20 -> 32 GPa over 0-4 km, +-5% a-b, 8 levels."""
    return ProblemConfig(name="config1_1025", ni=1025, nk=1025, mu_profile="layered",
                         amb_perturb=0.05, years=500.0,
                         mg=MGConfig(n_levels=8, nu_pre=2, nu_post=2, nu_coarse=32,
                                     tol_mode=1, tol=1e-9, max_cycles=200))


def config2() -> ProblemConfig:
    """4097x4097 stretched in depth: 4x finer rows over the 0-20 km fault
    zone (tanh transition centred at 21 km), config 0's friction with
    Dc = 2 mm, homogeneous mu = 30 GPa; FP32 V(2,2) cycles inside FP64
    refinement to a 1e-9 relative residual, 10 levels, 100 years."""
    return ProblemConfig(name="config2_4097", ni=4097, nk=4097, mu_profile="uniform", Dc_m=0.002,
                         years=100.0, stretch_ratio=4.0,
                         mg=MGConfig(n_levels=10, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1, tol=1e-9,
                                     max_cycles=200, precision=1, surface_prolong=1, coarse_solve=1))


def config1_mixed() -> ProblemConfig:
    c = config1()
    c.mg = dataclasses.replace(c.mg, precision=1)
    c.name = "config1_1025_mixed"
    return c


def small(n: int = 33, **kw) -> ProblemConfig:
    """A config-0-like problem on an n x n grid (n = 2^m + 1) for tests."""
    levels = 1
    m = n - 1
    while m % 2 == 0 and (m // 2) >= 8:
        m //= 2
        levels += 1
    c = ProblemConfig(name=f"small_{n}", ni=n, nk=n, mu_profile="uniform",
                      mg=MGConfig(n_levels=levels, nu_pre=2, nu_post=2, nu_coarse=32,
                                  tol_mode=1, tol=1e-10, max_cycles=200))
    return c.replace(**kw) if kw else c



def ensemble_instance(n: int, index: int, base_seed: int = 777) -> ProblemConfig:
    """Member `index` of the batched ensemble (config 4) on an n x n grid, with
    its parameters drawn from the seed base_seed + index: b - a in the
    seismogenic zone uniform in [0.002, 0.006] with a = 0.008, Dc log-uniform
    in [2, 20] mm, sigma_n uniform in [20, 80] MPa, seismogenic depth uniform
    in [10, 16] km, homogeneous mu uniform in [25, 35] GPa.  Mixed-precision
    multigrid with log2(n-1) - 1 levels (coarsest 5 x 5, solved exactly)."""
    import math
    import random
    rng = random.Random(base_seed + index)
    bma = rng.uniform(0.002, 0.006)
    dc = math.exp(rng.uniform(math.log(2e-3), math.log(20e-3)))
    sn = rng.uniform(20.0, 80.0)
    sd = rng.uniform(10.0, 16.0)
    mu = rng.uniform(25.0, 35.0)
    levels = int(round(math.log2(n - 1))) - 1
    return ProblemConfig(name=f"ensemble_{n}_{index}", ni=n, nk=n, mu_profile="uniform", mu_gpa=mu,
                         a_shallow=0.008, b=0.008 + bma, seis_depth_km=sd, taper_depth_km=sd + 4.0,
                         Dc_m=dc, sigma_n_mpa=sn, years=200.0, seed=base_seed + index,
                         mg=MGConfig(n_levels=levels, nu_pre=2, nu_post=2, nu_coarse=32, tol_mode=1,
                                     tol=1e-9, max_cycles=200, precision=1, surface_prolong=1,
                                     coarse_solve=1))

CONFIGS = {"config0": config0, "config1": config1, "config1_mixed": config1_mixed, "config2": config2}
