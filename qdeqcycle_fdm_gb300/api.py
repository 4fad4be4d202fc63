"""Python mirror of the reference's hot-path interface over the C ABI.

The reference's surface is the C++ free functions of ``functions.h:11-45``.
Here the same operations are methods of :class:`Solver` (one GB300 solver
with device-resident state), and :class:`Simulation` runs the reference's
``RK43`` loop (``odeSolver.cpp:1277-1674``) with the same start/step/state
shape as the CPU oracle, so parity tests read the same on both sides.

Every call goes through ``libqdeq_gb300.so``; nothing here computes on the
CPU.  Arrays follow the reference's layouts (ghosted ``(nz, nx)`` fields,
``nz``-long fault vectors).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import MgOptions, Rk43Params, Stats, Tuning, check
from .config import MGConfig

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _p(a):
    if a is None:
        return None
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("arrays must be C-contiguous float64")
    return a.ctypes.data_as(_dp)


def mg_options(mg: MGConfig) -> MgOptions:
    return MgOptions(mg.n_levels, mg.nu_pre, mg.nu_post, mg.nu_coarse, mg.tol_mode, mg.tol,
                     mg.max_cycles, mg.precision, mg.surface_prolong, mg.coarse_solve)


def ensemble_step(sims, nsteps: int = 1):
    """qd_ensemble_step over started Simulations (or Solvers): their GPU work
    interleaved; returns the steps each took."""
    solvers = [getattr(x, "solver", x) for x in sims]
    hs = (C.c_void_p * len(solvers))(*[s.h.value for s in solvers])
    done = (C.c_int * len(solvers))()
    check(_lib.load().qd_ensemble_step(hs, len(solvers), nsteps, done))
    return list(done)


def load_initial_u(path, ni: int, nk: int) -> np.ndarray:
    """The reference's initial-displacement file (odeSolver.cpp:96-128) as
    the ghosted (nk+2, ni+2) array U (ghosts zero)."""
    U = np.zeros((nk + 2, ni + 2))
    check(_lib.load().qd_load_initial_u(str(path).encode(), ni, nk, _p(U)))
    return U


def save_initial_u(path, U: np.ndarray) -> None:
    """Write U's interior in the layout load_initial_u reads."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    nk, ni = U.shape[0] - 2, U.shape[1] - 2
    check(_lib.load().qd_save_initial_u(str(path).encode(), ni, nk, _p(U)))


def set_medium(ni: int, nk: int, mu_node: np.ndarray) -> np.ndarray:
    """SetMedium's homogenisation on the GPU (odeSolver.cpp:337-589)."""
    L = _lib.load()
    me = np.zeros((2 * (nk + 2) - 1, 2 * (ni + 2) - 1))
    check(L.qd_set_medium(ni, nk, _p(np.ascontiguousarray(mu_node, dtype=np.float64)), _p(me)))
    return me


class Solver:
    """One device-resident solver: multigrid hierarchy + fault state."""

    def __init__(self, ni, nk, dh, mu_equi, mu_node, mg: MGConfig, jrow=None):
        """jrow: the depth metric of a stretched grid, J per staggered row of
        mu_equi (problem.depth_metric); None: the uniform grid."""
        self.L = _lib.load()
        self.ni, self.nk, self.nx, self.nz = ni, nk, ni + 2, nk + 2
        self.h = C.c_void_p()
        opt = mg_options(mg)
        jr = None if jrow is None else _p(np.ascontiguousarray(jrow, dtype=np.float64))
        check(self.L.qd_solver_create_mapped(ni, nk, dh, _p(np.ascontiguousarray(mu_equi)),
                                             _p(np.ascontiguousarray(mu_node)), jr, C.byref(opt),
                                             C.byref(self.h)))

    def close(self):
        if self.h:
            self.L.qd_solver_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stream_ptr(self) -> int:
        return int(self.L.qd_solver_stream(self.h) or 0)

    def set_options(self, mg: MGConfig):
        opt = mg_options(mg)
        check(self.L.qd_solver_set_options(self.h, C.byref(opt)))

    def stats(self) -> dict:
        st = Stats()
        check(self.L.qd_get_stats(self.h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in Stats._fields_}

    # -- displacement field ------------------------------------------------
    def upload_u(self, U):
        check(self.L.qd_upload_u(self.h, _p(np.ascontiguousarray(U))))

    def download_u(self, out=None):
        """The ghosted nz x nx field; `out`: a C-contiguous float64 array of
        that shape to write into (e.g. pinned host memory)."""
        U = np.zeros((self.nz, self.nx)) if out is None else out
        check(self.L.qd_download_u(self.h, _p(U)))
        return U

    def ode_solve(self):
        """multigrid() + extend_crew() on the device u; (cycles, ||r||, ||r0||)."""
        cyc = C.c_int(0)
        rn = C.c_double(0)
        r0 = C.c_double(0)
        check(self.L.qd_ode_solve(self.h, C.byref(cyc), C.byref(rn), C.byref(r0)))
        return cyc.value, rn.value, r0.value

    def ode_solve_host(self, U):
        """ode_solve with the reference's host round trip (U updated in place)."""
        cyc = C.c_int(0)
        rn = C.c_double(0)
        check(self.L.qd_ode_solve_host(self.h, _p(U), C.byref(cyc), C.byref(rn)))
        return cyc.value, rn.value

    def smooth(self, nsweeps):
        check(self.L.qd_mg_smooth(self.h, nsweeps))

    def vcycle(self):
        check(self.L.qd_mg_vcycle(self.h))

    def residual_norm(self):
        rn = C.c_double(0)
        check(self.L.qd_mg_residual_norm(self.h, C.byref(rn)))
        return rn.value

    KERNELS = {"down0": 0, "up0": 1, "residual": 2, "tail": 3}

    def time_kernel(self, name, reps=50):
        """Mean device microseconds per launch of one V-cycle kernel
        (qd_mg_time_kernel); perturbs the solver state."""
        us = C.c_double(0)
        check(self.L.qd_mg_time_kernel(self.h, self.KERNELS[name], reps, C.byref(us)))
        return us.value

    # -- fault -------------------------------------------------------------
    def fault_setup(self, prob, with_tau0=True):
        check(self.L.qd_fault_setup(self.h, _p(prob.a), _p(prob.b), _p(prob.eta), _p(prob.Tau_n0),
                                    _p(prob.SlipShift), _p(prob.tau0) if with_tau0 else None,
                                    prob.f0, prob.V0, prob.L, prob.Vini))

    def set_boundary(self, slip, t, ratio, dt):
        check(self.L.qd_set_boundary(self.h, _p(np.ascontiguousarray(slip)), t, ratio, dt))

    def eval_stress_on_fault(self):
        Ts = np.zeros(self.nz)
        Tn = np.zeros(self.nz)
        check(self.L.qd_eval_stress_on_fault(self.h, _p(Ts), _p(Tn)))
        return Ts, Tn

    def nrsearch(self, Ts, psi, V_seed):
        V = np.array(V_seed, dtype=np.float64, copy=True)
        iters = np.zeros(self.nz, dtype=np.int32)
        rc = self.L.qd_nrsearch(self.h, _p(np.ascontiguousarray(Ts)), _p(np.ascontiguousarray(psi)),
                                _p(V), iters.ctypes.data_as(_ip))
        return V, iters, rc

    def cal_dpsi(self, psi, V):
        d = np.zeros(self.nz)
        check(self.L.qd_cal_dpsi(self.h, _p(np.ascontiguousarray(psi)), _p(np.ascontiguousarray(V)),
                                 _p(d)))
        return d

    # -- RK43 --------------------------------------------------------------
    def rk43_start(self, prob):
        p = Rk43Params(prob.tmax, prob.ini_dt, prob.mindt, prob.maxdt, prob.totTol,
                       int(min(prob.maxNumSteps, 2**31 - 1)))
        check(self.L.qd_rk43_start(self.h, C.byref(p), _p(prob.Slip), _p(prob.psi)))

    def rk43_resume(self, prob, ck, params=None):
        """Restart from a fault-state checkpoint (Slip, psi, t, dt, errA0,
        errA1, it): the commit's refresh solve from the device u as it stands
        and the fault update.  `params`: (tmax, ini_dt, mindt, maxdt, totTol,
        maxNumSteps) overriding the problem's."""
        if params is None:
            params = (prob.tmax, prob.ini_dt, prob.mindt, prob.maxdt, prob.totTol,
                      int(min(prob.maxNumSteps, 2**31 - 1)))
        p = Rk43Params(*params)
        check(self.L.qd_rk43_resume(self.h, C.byref(p), _p(np.ascontiguousarray(ck["Slip"], dtype=np.float64)),
                                    _p(np.ascontiguousarray(ck["psi"], dtype=np.float64)), float(ck["t"]),
                                    float(ck["dt"]), float(ck["errA0"]), float(ck["errA1"]), int(ck["it"])))

    def probe_bounded_wait(self, polls):
        """qd_probe_bounded_wait: the return code and qd_last_error()."""
        rc = self.L.qd_probe_bounded_wait(self.h, int(polls))
        return rc, self.L.qd_last_error().decode(errors="replace")

    def rk43_step(self, n=1):
        done = C.c_int(0)
        check(self.L.qd_rk43_step(self.h, n, C.byref(done)))
        return done.value

    def rk43_state(self, out=None):
        """State after the last accepted step; `out`: a dict of nz float64
        arrays (Slip, psi, V, Ts, dpsi) to write into."""
        out = {k: np.zeros(self.nz) for k in ("Slip", "psi", "V", "Ts", "dpsi")} if out is None else out
        check(self.L.qd_rk43_get_state(self.h, _p(out["Slip"]), _p(out["psi"]), _p(out["V"]),
                                       _p(out["Ts"]), _p(out["dpsi"])))
        d = np.zeros(4)
        it = C.c_int(0)
        check(self.L.qd_rk43_get_scalars(self.h, _p(d), C.byref(it)))
        out.update(t=d[0], dt=d[1], errA=(d[2], d[3]), it=it.value)
        return out

    def rk43_set_state(self, Slip, psi, V, dpsi, t, dt, errA0, errA1, it):
        check(self.L.qd_rk43_set_state(self.h, _p(Slip), _p(psi), _p(V), _p(dpsi), t, dt, errA0,
                                       errA1, it))

    def rk43_step_host(self, n, st, U):
        """qd_rk43_step_host: n steps on a host-held state.  st: a dict of
        nz float64 arrays Slip, psi, V, dpsi, Ts and the scalars t, dt,
        errA, it (as rk43_state returns), updated in place; U: the ghosted
        nz x nx float64 field, updated in place.  Returns the steps taken."""
        d4 = np.array([st["t"], st["dt"], st["errA"][0], st["errA"][1]])
        it = C.c_int(int(st["it"]))
        done = C.c_int(0)
        check(self.L.qd_rk43_step_host(self.h, int(n), _p(st["Slip"]), _p(st["psi"]), _p(st["V"]), _p(st["dpsi"]),
                                       _p(st["Ts"]), _p(U), _p(d4), C.byref(it), C.byref(done)))
        st.update(t=d4[0], dt=d4[1], errA=(d4[2], d4[3]), it=it.value)
        return done.value

    def set_solution_history(self, m):
        """Start each stage solve from the least-squares combination of the
        last m solutions that best matches the new boundary data (m < 2: off,
        the previous solution as the reference)."""
        check(self.L.qd_set_solution_history(self.h, int(m)))

    def set_newton_start(self, mode):
        """Start of the Newton solve for slip rate: 0 the reference's x = 0
        (the default), 1 a binary32 solve of the equation's log form; the
        same FP64 iteration then ends at the same root in fewer steps."""
        check(self.L.qd_set_newton_start(self.h, int(mode)))

    def set_tail_sweeps(self, n):
        """Pre- and post-sweeps on the coarse tail's levels (<= 65 rows);
        0: the fine levels' schedule (the default)."""
        check(self.L.qd_set_tail_sweeps(self.h, int(n)))

    def set_smooth_correction(self, ratio):
        """Mixed precision: a level-0 smoothing pass instead of a V-cycle
        after a cycle that left ||r|| within `ratio` of the threshold (0:
        off, the default)."""
        check(self.L.qd_set_smooth_correction(self.h, float(ratio)))

    def autotune(self, reps=3):
        """Time the candidate smoother schedules and tile box widths on this
        solver's problem (the last stored solve replayed from the solution
        history's guess when the history holds three solutions, else solves
        from a zero interior; to its tolerance), keep the fastest, restore u;
        returns the qd_tuning fields."""
        t = Tuning()
        check(self.L.qd_autotune(self.h, int(reps), C.byref(t)))
        return {f: getattr(t, f) for f, _ in Tuning._fields_}

    def set_tiles(self, box_up=0, box_down=0):
        check(self.L.qd_set_tiles(self.h, int(box_up), int(box_down)))

    def solution_history_fit(self):
        """(coefficients in use, boundary misfit / change) of the last fit."""
        c = np.zeros(8)
        nd = C.c_int(0)
        check(self.L.qd_solution_history_fit(self.h, _p(c), C.byref(nd)))
        return c[:nd.value].copy(), float(c[7])

    # -- files -------------------------------------------------------------
    def snapshot(self, path, full=True, asynchronous=False):
        """The reference's snapshot record of the current state (qd_snapshot)."""
        check(self.L.qd_snapshot(self.h, str(path).encode(), int(full), int(asynchronous)))

    def snapshot_wait(self):
        check(self.L.qd_snapshot_wait(self.h))

    def checkpoint_save(self, path):
        check(self.L.qd_checkpoint_save(self.h, str(path).encode()))

    def checkpoint_load(self, path):
        check(self.L.qd_checkpoint_load(self.h, str(path).encode()))


class Simulation:
    """RK43 on the GPU with the oracle's start/step/state interface."""

    def __init__(self, prob, mg: MGConfig, with_tau0=True):
        self.prob = prob
        self.solver = Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, mg,
                             jrow=getattr(prob, "jrow", None))
        self.solver.fault_setup(prob, with_tau0=with_tau0)
        self.solver.upload_u(prob.U)

    def start(self):
        self.solver.rk43_start(self.prob)
        return 0

    def resume(self, ck, U=None, params=None):
        """Restart from a fault-state checkpoint; U (ghosted) is the refresh
        solve's guess (default: the problem's initial U)."""
        self.solver.upload_u(self.prob.U if U is None else U)
        self.solver.rk43_resume(self.prob, ck, params)
        return 0

    def step(self, n=1):
        return self.solver.rk43_step(n)

    def state(self, with_u=True):
        st = self.solver.rk43_state()
        if with_u:
            st["U"] = self.solver.download_u()
        st.update(self.solver.stats())
        return st

    def close(self):
        self.solver.close()
