"""Synthetic problem set-up: medium, friction, prestress and initial state.

Arrays use the reference's layouts (see ``struct.h:49-139`` and
``Alloc.cpp:3-42``): ghosted fields are ``(nz, nx)`` with ``nx = ni + 2``,
``nz = nk + 2``; fault vectors are ``nz`` long with valid entries ``1..nk``;
the homogenised face moduli ``mu_equi`` are ``(2nz-1, 2nx-1)``.

Geometry follows ``coord.cpp:18,27``: ghosted column ``i`` sits at
``x = (i-1) dh`` and ghosted row ``k`` at depth ``(nk - k) dh``, so compact
row 0 is the deepest row and compact row ``nk-1`` the free surface; the
fault is compact column 0 and the remote boundary compact column ``ni-1``.

Friction set-up follows ``fault.cpp:85-127``: ``psi0 = f0 + b ln(V0/Vp)``,
``eta = sqrt(rho mu)/2``, ``Slip = 2 u(fault)``, ``SlipShift = u(far)``.
The reference has no prestress term; ``tau0`` (added to the stress the
Newton solve sees) is chosen so that ``V = Vp`` at ``t = 0`` with ``u = 0``.
With ``prestress=False`` it is zero and the set-up reduces to the reference's.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np

from .config import YEAR_S, ProblemConfig


@dataclass
class Problem:
    cfg: ProblemConfig
    ni: int
    nk: int
    nx: int
    nz: int
    dh: float
    mu_node: np.ndarray
    rho: np.ndarray
    mu_equi: np.ndarray
    a: np.ndarray
    b: np.ndarray
    eta: np.ndarray
    Tau_n0: np.ndarray
    SlipShift: np.ndarray
    tau0: np.ndarray
    Slip: np.ndarray
    psi: np.ndarray
    U: np.ndarray
    f0: float
    V0: float
    L: float
    Vini: float
    tmax: float
    ini_dt: float
    mindt: float
    maxdt: float
    totTol: float
    maxNumSteps: int
    jrow: Optional[np.ndarray] = None   # depth metric per staggered row (stretched grids)


def depth_of_rows(nk: int, dh: float) -> np.ndarray:
    """Depth (m) of every ghosted row k = 0..nk+1 (coord.cpp:27)."""
    return (nk - np.arange(nk + 2, dtype=np.float64)) * dh


def _lncosh(x):
    a = np.abs(x)
    return a + np.log1p(np.exp(-2.0 * a)) - np.log(2.0)


def depth_metric(cfg: ProblemConfig):
    """A grid stretched in depth (the reference's is uniform, coord.cpp:18,27).

    In the normalised depth xi in [0, 1] (0 at the surface) the row spacing
    grows smoothly by cfg.stretch_ratio = R across a tanh transition:
        d(xi) = D g(xi) / g(1),   g'(xi) = 1 + (R - 1) (1 + tanh((xi - xi0) / w)) / 2,
        g(xi) = xi + (R - 1) / 2 [xi + w (lncosh((xi - xi0) / w) - lncosh(-xi0 / w))],
    with w = cfg.stretch_width and xi0 placing the transition's centre at
    cfg.stretch_depth_km.  The computational coordinate zeta = D xi has the
    same uniform spacing as x, and the metric is J = dz/dzeta = g'(xi) / g(1).

    Returns (depth of every ghosted row k = 0..nk+1 in m, J at every
    staggered row r = 0..2nz-2 of mu_equi).  Ghosted row k is compact row
    k - 1 at xi = 1 - (k - 1) / (nk - 1); staggered row r sits at compact
    position r / 2 - 1.  The ghost rows' J mirrors the interior's about the
    first and last rows, as the mirrored (Neumann) rows of the operator do.
    """
    nk = cfg.nk
    D = cfg.domain_m
    R, w = cfg.stretch_ratio, cfg.stretch_width

    def g(xi, xi0):
        return xi + 0.5 * (R - 1.0) * (xi + w * (_lncosh((xi - xi0) / w) - _lncosh(-xi0 / w)))

    frac = cfg.stretch_depth_km * 1e3 / D
    lo, hi = 0.0, 1.0
    for _ in range(200):                    # g(xi0, xi0) / g(1, xi0) = frac, by bisection
        mid = 0.5 * (lo + hi)
        if g(mid, mid) / g(1.0, mid) < frac:
            lo = mid
        else:
            hi = mid
    xi0 = 0.5 * (lo + hi)
    g1 = g(1.0, xi0)
    n1 = nk - 1
    k = np.arange(nk + 2, dtype=np.float64)
    depth = D * g(1.0 - (k - 1.0) / n1, xi0) / g1
    p = np.arange(2 * (nk + 2) - 1, dtype=np.float64) / 2.0 - 1.0
    p = np.where(p < 0.0, -p, p)
    p = np.where(p > n1, 2.0 * n1 - p, p)
    xi = 1.0 - p / n1
    jrow = (1.0 + 0.5 * (R - 1.0) * (1.0 + np.tanh((xi - xi0) / w))) / g1
    return depth, np.ascontiguousarray(jrow)


def mu_profile(cfg: ProblemConfig, depth_m: np.ndarray) -> np.ndarray:
    if cfg.mu_profile == "uniform":
        return np.full_like(depth_m, cfg.mu_gpa)
    if cfg.mu_profile == "layered":
        dkm = np.clip(depth_m * 1e-3, 0.0, None)
        frac = np.clip(dkm / cfg.layer_depth_km, 0.0, 1.0)
        return cfg.mu_surface_gpa + (cfg.mu_deep_gpa - cfg.mu_surface_gpa) * frac
    raise ValueError(f"unknown mu profile {cfg.mu_profile!r}")


def a_profile(cfg: ProblemConfig, depth_m: np.ndarray) -> np.ndarray:
    dkm = depth_m * 1e-3
    a = np.where(dkm <= cfg.seis_depth_km, cfg.a_shallow, cfg.a_deep)
    ramp = (dkm > cfg.seis_depth_km) & (dkm < cfg.taper_depth_km)
    t = (dkm - cfg.seis_depth_km) / (cfg.taper_depth_km - cfg.seis_depth_km)
    return np.where(ramp, cfg.a_shallow + (cfg.a_deep - cfg.a_shallow) * t, a)


def build_problem(cfg: ProblemConfig,
                  homogenize: Optional[Callable[[int, int, np.ndarray], np.ndarray]] = None
                  ) -> Problem:
    """Assemble every input array of one simulation.

    ``homogenize(ni, nk, mu_node) -> mu_equi`` computes the face moduli
    (the reference's SetMedium); by default the product's GPU kernel does it.
    """
    ni, nk = cfg.ni, cfg.nk
    nx, nz = ni + 2, nk + 2
    dh = cfg.dh
    jrow = None
    if cfg.stretch_ratio != 1.0:
        depth, jrow = depth_metric(cfg)
    else:
        depth = depth_of_rows(nk, dh)
    mu_rows = mu_profile(cfg, depth)
    mu_node = np.ascontiguousarray(np.repeat(mu_rows[:, None], nx, axis=1))
    rho = mu_node / (cfg.cs_kms ** 2)
    if homogenize is None:
        from . import api
        homogenize = api.set_medium
    mu_equi = np.ascontiguousarray(homogenize(ni, nk, mu_node))

    a = np.zeros(nz)
    b = np.zeros(nz)
    a[1:nk + 1] = a_profile(cfg, depth[1:nk + 1])
    b[1:nk + 1] = cfg.b
    if cfg.amb_perturb:
        rng = np.random.default_rng(cfg.seed)
        w = rng.uniform(-1.0, 1.0, size=nk)       # fault node order k = 1..nk
        amb = a[1:nk + 1] - b[1:nk + 1]
        a[1:nk + 1] = b[1:nk + 1] + amb * (1.0 + cfg.amb_perturb * w)
    eta = np.zeros(nz)
    eta[1:nk + 1] = 0.5 * np.sqrt(rho[1:nk + 1, 1] * mu_node[1:nk + 1, 1])
    Tau_n0 = np.zeros(nz)
    Tau_n0[1:nk + 1] = -cfg.sigma_n_mpa
    psi = np.zeros(nz)
    psi[1:nk + 1] = cfg.f0 + b[1:nk + 1] * np.log(cfg.V0 / cfg.Vp)
    tau0 = np.zeros(nz)
    if cfg.prestress:
        k = slice(1, nk + 1)
        tau0[k] = (cfg.sigma_n_mpa * a[k] *
                   np.arcsinh(cfg.Vp / (2.0 * cfg.V0) * np.exp(psi[k] / a[k])) + eta[k] * cfg.Vp)
    U = np.zeros((nz, nx))
    Slip = np.zeros(nz)
    Slip[1:nk + 1] = 2.0 * U[1:nk + 1, 1]
    SlipShift = np.ascontiguousarray(U[:, ni].copy())
    return Problem(cfg=cfg, ni=ni, nk=nk, nx=nx, nz=nz, dh=dh, mu_node=mu_node, rho=rho,
                   mu_equi=mu_equi, a=a, b=b, eta=eta, Tau_n0=Tau_n0, SlipShift=SlipShift,
                   tau0=tau0, Slip=Slip, psi=psi, U=U, f0=cfg.f0, V0=cfg.V0, L=cfg.Dc_m,
                   Vini=cfg.Vp, tmax=cfg.years * YEAR_S, ini_dt=cfg.ini_dt, mindt=cfg.mindt,
                   maxdt=cfg.maxdt, totTol=cfg.totTol, maxNumSteps=cfg.maxNumSteps, jrow=jrow)
