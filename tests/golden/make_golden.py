"""Generate golden vectors from the reference's own host functions.

Builds ``oracle/_ref/libref_host.so`` from the reference sources (the recipe
is ``oracle/Makefile``; it compiles fault.cpp, Alloc.cpp and odeSolver.cpp
in place) and records the outputs of ``eval_stress_on_fault``, ``NRsearch``,
``cal_dpsi``, ``computeError``, ``computeStepSize``, ``setBoundary``,
``extend_crew``, ``interp_2d`` and ``interp2_2d`` on seeded inputs into
``ref_host_golden.npz`` next to this script.

Run here, where the reference sources exist:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402


def _p(a):
    return oracle._p(a)


def main():
    oracle.build(ref=True)
    R = oracle.ref_host()
    if R is None:
        raise SystemExit("reference host library could not be built")
    rng = np.random.default_rng(20261203)
    out = {}

    # --- eval_stress_on_fault (fault.cpp:139-164) ---
    ni, nk = 17, 33
    nx, nz = ni + 2, nk + 2
    dh = 312.5
    U = rng.normal(size=(nz, nx)) * 0.1
    mu_node = rng.uniform(20.0, 36.0, size=(nz, nx))
    Tau_n0 = -rng.uniform(20.0, 80.0, size=nz)
    Ts = np.zeros(nz)
    Tn = np.zeros(nz)
    R.ref_eval_stress_on_fault(ni, nk, dh, _p(U), _p(mu_node), _p(Tau_n0), _p(Ts), _p(Tn))
    out.update(stress_ni=ni, stress_nk=nk, stress_dh=dh, stress_U=U, stress_mu=mu_node,
               stress_Tau_n0=Tau_n0, stress_Ts=Ts, stress_Tn=Tn)

    # --- NRsearch (fault.cpp:169-232): interseismic to coseismic slip rates ---
    nk = 200
    nz = nk + 2
    a = np.zeros(nz)
    eta = np.zeros(nz)
    psi = np.zeros(nz)
    Tn = np.zeros(nz)
    Ts = np.zeros(nz)
    V = np.zeros(nz)
    k = slice(1, nk + 1)
    a[k] = rng.uniform(0.006, 0.03, nk)
    eta[k] = rng.uniform(2.0, 6.0, nk)
    Tn[k] = -rng.uniform(20.0, 80.0, nk)
    logV = rng.uniform(-12.0, 0.5, nk)            # target slip rates 1e-12 .. 3 m/s
    psi[k] = 0.6 + 0.012 * np.log(1e-6 / 10.0 ** rng.uniform(-12, -3, nk))
    Vt = 10.0 ** logV
    Ts[k] = (-Tn[k]) * a[k] * np.arcsinh(Vt / 2e-6 * np.exp(psi[k] / a[k])) + eta[k] * Vt
    seeds = np.zeros(nz)
    seeds[k] = np.where(rng.uniform(size=nk) < 0.5, 0.0, 10.0 ** rng.uniform(-12, 0, nk))
    V[:] = seeds
    R.ref_nrsearch(nk, _p(Ts), _p(Tn), _p(a), _p(eta), _p(psi), 1e-6, _p(V))
    out.update(nr_nk=nk, nr_Ts=Ts, nr_Tn=Tn, nr_a=a, nr_eta=eta, nr_psi=psi, nr_seed=seeds, nr_V=V)

    # --- cal_dpsi (odeSolver.cpp:1190-1206), including b <= 1e-3 and exp overflow ---
    nk = 64
    nz = nk + 2
    psi = rng.uniform(0.4, 0.9, nz)
    b = rng.uniform(0.0, 0.03, nz)
    b[5] = 1e-3
    b[6] = 1e-5
    psi[7] = -20.0           # exp((f0-psi)/b) overflows
    V = 10.0 ** rng.uniform(-12, 0, nz)
    dpsi = np.zeros(nz)
    R.ref_cal_dpsi(nk, _p(psi), _p(b), _p(V), 0.6, 1e-6, 0.008, _p(dpsi))
    out.update(dp_nk=nk, dp_psi=psi, dp_b=b, dp_V=V, dp_out=dpsi)

    # --- computeError (odeSolver.cpp:1211-1238) ---
    nk = 129
    nz = nk + 2
    s3, p3, s4, p4 = (rng.normal(size=nz) for _ in range(4))
    out.update(err_nk=nk, err_s3=s3, err_p3=p3, err_s4=s4, err_p4=p4,
               err_out=np.array(R.ref_compute_error(nk, _p(s3), _p(p3), _p(s4), _p(p4))))

    # --- computeStepSize (odeSolver.cpp:1241-1271) ---
    cases = []
    for it in (0, 1, 3, 4, 5, 50):
        for dt in (1e-3, 1.0, 3e7):
            for tot in (1e-12, 1e-9, 1e-7, 3e-7, 1e-3):
                errA = np.array([10.0 ** rng.uniform(-10, -6), 10.0 ** rng.uniform(-10, -6)])
                val = R.ref_compute_step_size(it, dt, 1e-5, 1e8, tot, 1e-7, _p(errA))
                cases.append([it, dt, tot, errA[0], errA[1], val])
    out["ss_cases"] = np.array(cases)

    # --- setBoundary (odeSolver.cpp:1150-1188) / extend_crew (:612-650) ---
    ni, nk = 9, 17
    nx, nz = ni + 2, nk + 2
    U = rng.normal(size=(nz, nx))
    slip = rng.normal(size=nz)
    shift = rng.normal(size=nz)
    Ub = U.copy()
    R.ref_set_boundary(ni, nk, _p(Ub), _p(slip), _p(shift), 1e-9, 3.2e9, 0.62, 1.7e6)
    Ue = U.copy()
    R.ref_extend_crew(ni, nk, _p(Ue))
    out.update(bc_ni=ni, bc_nk=nk, bc_U=U, bc_slip=slip, bc_shift=shift, bc_out=Ub, ec_out=Ue)

    # --- interp_2d / interp2_2d (odeSolver.cpp:134-268) ---
    pts = []
    for _ in range(64):
        z = rng.uniform(5.0, 40.0, 12)
        xi, yi = rng.uniform(-0.5, 0.5, 2)
        pts.append(np.concatenate([z, [xi, yi, R.ref_interp_2d(_p(z), xi, yi),
                                       R.ref_interp2_2d(_p(z), xi, yi)]]))
    out["interp"] = np.array(pts)

    path = os.path.join(HERE, "ref_host_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
