"""ctypes bindings of the CPU oracle (qdeq_oracle.c) and of the reference-built
checkers in ``oracle/_ref``.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py`` (its ``cpu_baseline`` leg and the ``--impl reference`` arm) import
this package; the product package never does.

Array conventions follow the reference (QDEqCycle_FDM):
  * ghosted fields ``U``/``mu_node``: shape ``(nz, nx)`` float64, ``nx = ni+2``,
    ``nz = nk+2`` (index ``i + k*nx``, struct.h:49-72);
  * compact multigrid fields: shape ``(N, K) = (nk, ni)``;
  * ``mu_equi``: shape ``(2*nz-1, 2*nx-1)``;
  * fault vectors: length ``nz``, valid entries ``1..nk``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libqdeq_oracle.so")
_REF_HOST = os.path.join(_HERE, "_ref", "libref_host.so")
REF_KERNELS_CUBIN = os.path.join(_HERE, "_ref", "ref_kernels.cubin")
REF_DIR = "/root/reference"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build(ref: bool | None = None) -> None:
    """Compile the oracle (and, if the reference sources exist, _ref/)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    if ref is None:
        ref = os.path.isdir(REF_DIR)
    if ref:
        subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF_DIR={REF_DIR}"], check=True)


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(_dp)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build(ref=False)
        L = C.CDLL(_LIB_PATH)
        L.qo_sim_create.restype = C.c_void_p
        L.qo_sim_create.argtypes = [C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]
        L.qo_sim_free.argtypes = [C.c_void_p]
        L.qo_sim_set_fault.argtypes = [C.c_void_p] + [_dp] * 8 + [C.c_double] * 4
        L.qo_sim_set_params.argtypes = [C.c_void_p] + [C.c_double] * 5 + [C.c_int]
        L.qo_sim_set_U.argtypes = [C.c_void_p, _dp]
        L.qo_sim_set_surface_prolong.argtypes = [C.c_void_p, C.c_int]
        L.qo_sim_set_coarse_solve.argtypes = [C.c_void_p, C.c_int]
        L.qo_sim_set_metric.argtypes = [C.c_void_p, _dp]
        L.qo_sim_start.argtypes = [C.c_void_p]
        L.qo_sim_step.argtypes = [C.c_void_p]
        L.qo_sim_resume.argtypes = [C.c_void_p, _dp, _dp] + [C.c_double] * 4 + [C.c_int]
        L.qo_sim_get.argtypes = [C.c_void_p] + [_dp] * 6
        L.qo_sim_scalars.argtypes = [C.c_void_p, _dp, C.POINTER(C.c_longlong)]
        L.qo_sim_set_scalars.argtypes = [C.c_void_p] + [C.c_double] * 4 + [C.c_int]
        L.qo_compute_error.restype = C.c_double
        L.qo_compute_step_size.restype = C.c_double
        L.qo_compute_step_size.argtypes = [C.c_int] + [C.c_double] * 5 + [_dp]
        L.qo_compute_error.argtypes = [C.c_int] + [_dp] * 4
        L.qo_nrsearch.argtypes = [C.c_int] + [_dp] * 6 + [C.c_double, _dp, _ip]
        L.qo_cal_dpsi.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double, _dp]
        L.qo_eval_stress_on_fault.argtypes = [C.c_int, C.c_int, C.c_double] + [_dp] * 5
        L.qo_set_boundary.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp] + [C.c_double] * 4
        L.qo_extend_crew.argtypes = [C.c_int, C.c_int, _dp]
        L.qo_set_medium.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
        L.qo_set_threads.argtypes = [C.c_int]
        for fn in (L.qo_interp_xedge, L.qo_interp_zedge):
            fn.restype = C.c_double
            fn.argtypes = [_dp, C.c_double, C.c_double]
        _lib = L
    return _lib


def ref_host():
    """The reference's own host functions (built from its sources), or None."""
    if not os.path.exists(_REF_HOST):
        return None
    L = C.CDLL(_REF_HOST)
    L.ref_eval_stress_on_fault.argtypes = [C.c_int, C.c_int, C.c_double] + [_dp] * 5
    L.ref_nrsearch.argtypes = [C.c_int] + [_dp] * 5 + [C.c_double, _dp]
    L.ref_cal_dpsi.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double, _dp]
    L.ref_compute_error.restype = C.c_double
    L.ref_compute_error.argtypes = [C.c_int] + [_dp] * 4
    L.ref_compute_step_size.restype = C.c_double
    L.ref_compute_step_size.argtypes = [C.c_int] + [C.c_double] * 5 + [_dp]
    L.ref_set_boundary.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp] + [C.c_double] * 4
    L.ref_extend_crew.argtypes = [C.c_int, C.c_int, _dp]
    L.ref_interp_2d.restype = C.c_double
    L.ref_interp_2d.argtypes = [_dp, C.c_double, C.c_double]
    L.ref_interp2_2d.restype = C.c_double
    L.ref_interp2_2d.argtypes = [_dp, C.c_double, C.c_double]
    return L


def set_threads(n: int) -> None:
    lib().qo_set_threads(int(n))


# --------------------------------------------------------------------------
# multigrid restated kernels (stateful wrapper over qo_mg)
# --------------------------------------------------------------------------
class _QoMg(C.Structure):
    _fields_ = [("n_levels", C.c_int), ("nu_pre", C.c_int), ("nu_post", C.c_int),
                ("nu_coarse", C.c_int), ("N", C.c_int * 16), ("K", C.c_int * 16),
                ("fc", C.c_int * 16), ("DH", C.c_double * 16), ("nx", C.c_int),
                ("mu", _dp), ("mux", _dp), ("muz", _dp), ("own_x", _dp), ("own_z", _dp),
                ("res", _dp * 16), ("res2", _dp * 16), ("err2", _dp * 16),
                ("delta", _dp), ("rowsum", _dp), ("surface_prolong", C.c_int),
                ("coarse_solve", C.c_int)]


class Multigrid:
    """The reference's multigrid (odeSolver.cpp:652-1147) on the CPU."""

    def __init__(self, ni, nk, dh, mu_equi, n_levels=6, nu_pre=32, nu_post=32, nu_coarse=32,
                 surface_prolong=0, coarse_solve=0, jrow=None):
        L = lib()
        self._mu = np.ascontiguousarray(mu_equi, dtype=np.float64)
        self.m = _QoMg()
        rc = L.qo_mg_init(C.byref(self.m), ni, nk, C.c_double(dh), _p(self._mu), n_levels,
                          nu_pre, nu_post, nu_coarse)
        if rc != 0:
            raise ValueError("bad multigrid configuration")
        self.m.surface_prolong = int(surface_prolong)
        self.m.coarse_solve = int(coarse_solve)
        if jrow is not None:
            self._jrow = np.ascontiguousarray(jrow, dtype=np.float64)
            L.qo_mg_set_metric(C.byref(self.m), nk, _p(self._jrow))
        self.ni, self.nk = ni, nk
        self.shapes = [(self.m.N[l], self.m.K[l]) for l in range(n_levels)]

    def __del__(self):
        try:
            lib().qo_mg_free(C.byref(self.m))
        except Exception:
            pass

    def rbgs(self, u, f, level, phase):
        lib().qo_rbgs(C.byref(self.m), _p(u), _p(f), level, phase)

    def residual(self, r, u, f, level):
        lib().qo_residual(C.byref(self.m), _p(r), _p(u), _p(f), level)

    def restriction(self, r2, r, e2, level):
        lib().qo_restriction(C.byref(self.m), _p(r2), _p(r), _p(e2), level)

    def prolongate(self, u, e2, level):
        lib().qo_prolongate(C.byref(self.m), _p(u), _p(e2), level)

    def vcycle(self, u, f, level=0):
        lib().qo_vcycle(C.byref(self.m), _p(u), _p(f), level)

    def norm2(self, r, level=0):
        f = lib().qo_norm2
        f.restype = C.c_double
        return f(C.byref(self.m), _p(r), level)

    def r0_norm(self, u, level=0):
        f = lib().qo_r0_norm
        f.restype = C.c_double
        return f(C.byref(self.m), _p(u), level)

    def solve(self, u, f=None, tol_mode=0, tol=1e-9, max_cycles=0):
        """multigrid(); returns (cycles, rnorm, r0norm)."""
        if f is None:
            f = np.zeros_like(u)
        rn = C.c_double(0.0)
        r0 = C.c_double(0.0)
        fn = lib().qo_multigrid
        fn.restype = C.c_int
        cyc = fn(C.byref(self.m), _p(u), _p(f), tol_mode, C.c_double(tol), max_cycles,
                 C.byref(rn), C.byref(r0))
        return cyc, rn.value, r0.value


# --------------------------------------------------------------------------
# fault physics / boundary
# --------------------------------------------------------------------------
def eval_stress_on_fault(ni, nk, dh, U, mu_node, Tau_n0):
    nz = nk + 2
    Ts = np.zeros(nz)
    Tn = np.zeros(nz)
    lib().qo_eval_stress_on_fault(ni, nk, C.c_double(dh), _p(U), _p(mu_node), _p(Tau_n0),
                                  _p(Ts), _p(Tn))
    return Ts, Tn


def nrsearch(nk, Ts, Tn, a, eta, psi, V0, V_seed, tau0=None):
    V = np.array(V_seed, dtype=np.float64, copy=True)
    iters = np.zeros(nk + 2, dtype=np.int32)
    st = lib().qo_nrsearch(nk, _p(Ts), _p(Tn), _p(tau0), _p(a), _p(eta), _p(psi),
                           C.c_double(V0), _p(V), iters.ctypes.data_as(_ip))
    return V, iters, st


def cal_dpsi(nk, psi, b, V, f0, V0, L):
    d = np.zeros(nk + 2)
    lib().qo_cal_dpsi(nk, _p(psi), _p(b), _p(V), C.c_double(f0), C.c_double(V0),
                      C.c_double(L), _p(d))
    return d


def set_boundary(ni, nk, U, slip, slip_shift, vini, t, ratio, dt):
    lib().qo_set_boundary(ni, nk, _p(U), _p(slip), _p(slip_shift), C.c_double(vini),
                          C.c_double(t), C.c_double(ratio), C.c_double(dt))


def extend_crew(ni, nk, U):
    lib().qo_extend_crew(ni, nk, _p(U))


def set_medium(ni, nk, mu_node):
    """SetMedium homogenisation; returns (mu_half, mu_equi)."""
    nx, nz = ni + 2, nk + 2
    mh = np.zeros((2 * nz - 1, 2 * nx - 1))
    me = np.zeros((2 * nz - 1, 2 * nx - 1))
    lib().qo_set_medium(ni, nk, _p(np.ascontiguousarray(mu_node)), _p(mh), _p(me))
    return mh, me


def compute_error(nk, s3, p3, s4, p4):
    return lib().qo_compute_error(nk, _p(s3), _p(p3), _p(s4), _p(p4))


def compute_step_size(it, dt, mindt, maxdt, totErr, totTol, errA):
    e = np.asarray(errA, dtype=np.float64).copy()
    return lib().qo_compute_step_size(it, dt, mindt, maxdt, totErr, totTol, _p(e))


# --------------------------------------------------------------------------
# the whole RK43 run
# --------------------------------------------------------------------------
class Simulation:
    """The reference's RK43 loop (odeSolver.cpp:1277-1674) on the CPU."""

    def __init__(self, prob, n_levels=6, nu_pre=32, nu_post=32, nu_coarse=32, tol_mode=0,
                 tol=1e-9, max_cycles=0, surface_prolong=0, coarse_solve=0):
        L = lib()
        self.prob = prob
        self.ni, self.nk = prob.ni, prob.nk
        self._keep = [np.ascontiguousarray(prob.mu_node), np.ascontiguousarray(prob.mu_equi)]
        self.h = L.qo_sim_create(prob.ni, prob.nk, C.c_double(prob.dh), _p(self._keep[0]),
                                 _p(self._keep[1]), n_levels, nu_pre, nu_post, nu_coarse,
                                 tol_mode, C.c_double(tol), max_cycles)
        L.qo_sim_set_fault(self.h, _p(prob.a), _p(prob.b), _p(prob.eta), _p(prob.Tau_n0),
                           _p(prob.SlipShift), _p(prob.tau0), _p(prob.Slip), _p(prob.psi),
                           C.c_double(prob.f0), C.c_double(prob.V0), C.c_double(prob.L),
                           C.c_double(prob.Vini))
        L.qo_sim_set_params(self.h, prob.tmax, prob.ini_dt, prob.mindt, prob.maxdt,
                            prob.totTol, int(prob.maxNumSteps))
        L.qo_sim_set_U(self.h, _p(np.ascontiguousarray(prob.U)))
        L.qo_sim_set_surface_prolong(self.h, int(surface_prolong))
        L.qo_sim_set_coarse_solve(self.h, int(coarse_solve))
        jrow = getattr(prob, "jrow", None)
        if jrow is not None:          # a grid stretched in depth
            self._keep.append(np.ascontiguousarray(jrow, dtype=np.float64))
            L.qo_sim_set_metric(self.h, _p(self._keep[-1]))

    def __del__(self):
        try:
            lib().qo_sim_free(self.h)
        except Exception:
            pass

    def start(self):
        return lib().qo_sim_start(self.h)

    def step(self):
        return lib().qo_sim_step(self.h)

    def state(self):
        nx, nz = self.ni + 2, self.nk + 2
        U = np.zeros((nz, nx))
        out = {k: np.zeros(nz) for k in ("Slip", "psi", "V", "Ts", "dpsi")}
        lib().qo_sim_get(self.h, _p(U), _p(out["Slip"]), _p(out["psi"]), _p(out["V"]),
                         _p(out["Ts"]), _p(out["dpsi"]))
        out["U"] = U
        d = np.zeros(4)
        iv = (C.c_longlong * 6)()
        lib().qo_sim_scalars(self.h, _p(d), iv)
        out.update(t=d[0], dt=d[1], errA=(d[2], d[3]), it=iv[0], solves=iv[1], vcycles=iv[2],
                   attempts=iv[3], newton_iters=iv[4], status=iv[5])
        return out

    def set_scalars(self, t, dt, errA0, errA1, it):
        lib().qo_sim_set_scalars(self.h, t, dt, errA0, errA1, it)

    def set_params(self, tmax, ini_dt, mindt, maxdt, totTol, maxNumSteps):
        lib().qo_sim_set_params(self.h, tmax, ini_dt, mindt, maxdt, totTol, int(maxNumSteps))

    def set_U(self, U):
        lib().qo_sim_set_U(self.h, _p(np.ascontiguousarray(U, dtype=np.float64)))

    def resume(self, ck, U=None):
        """Restart from a fault-state checkpoint (a dict with Slip, psi, t, dt,
        errA0, errA1, it): the refresh solve from U (default: the current U)
        and the fault update that end an accepted step."""
        if U is not None:
            self.set_U(U)
        return lib().qo_sim_resume(self.h, _p(np.ascontiguousarray(ck["Slip"], dtype=np.float64)),
                                   _p(np.ascontiguousarray(ck["psi"], dtype=np.float64)),
                                   float(ck["t"]), float(ck["dt"]), float(ck["errA0"]),
                                   float(ck["errA1"]), int(ck["it"]))


# --------------------------------------------------------------------------
# the reference's own GPU multigrid (refgpu.c over _ref/ref_kernels.cubin)
# --------------------------------------------------------------------------
_REFGPU_PATH = os.path.join(_HERE, "_build", "librefgpu.so")
_SOLVE_HOOK = C.CFUNCTYPE(C.c_int, C.c_void_p, _dp, C.c_int, C.c_int, _dp)


def refgpu_available() -> bool:
    return os.path.exists(_REFGPU_PATH) and os.path.exists(REF_KERNELS_CUBIN)


class RefGpuMultigrid:
    """The reference's multigrid() on the GPU: its unmodified kernels with
    the host sequencing restated in C (odeSolver.cpp:652-755, 1101-1147):
    6 levels, V(32,32), u up and down every solve, a blocking norm per
    V-cycle.  attach(sim) makes an oracle Simulation call it for every
    elliptic solve, so the RK43 loop runs as the reference program does:
    host code around GPU multigrid.  rel = 1 stops at tol * ||r0|| (the
    relative tolerance of the solvers it is compared with), rel = 0 at the
    reference's absolute tol."""

    def __init__(self, prob, rel=1, tol=1e-9):
        L = C.CDLL(_REFGPU_PATH)
        L.rg_create.restype = C.c_void_p
        L.rg_create.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_double, _dp, C.c_int, C.c_double,
                                C.c_char_p, C.c_int]
        L.rg_free.argtypes = [C.c_void_p]
        L.rg_stats.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
        self.L = L
        self._mu = np.ascontiguousarray(prob.mu_equi, dtype=np.float64)
        err = C.create_string_buffer(256)
        self.h = L.rg_create(REF_KERNELS_CUBIN.encode(), prob.ni, prob.nk, prob.dh, _p(self._mu), int(rel),
                             float(tol), err, 256)
        if not self.h:
            raise RuntimeError(f"reference GPU multigrid: {err.value.decode()}")
        self.hook = C.cast(L.rg_solve, C.c_void_p).value

    def attach(self, sim):
        fn = lib().qo_sim_set_solve_hook
        fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        fn(sim.h, self.hook, self.h)

    def stats(self):
        v = (C.c_longlong * 2)()
        self.L.rg_stats(self.h, v)
        return {"solves": v[0], "vcycles": v[1]}

    def close(self):
        if self.h:
            self.L.rg_free(self.h)
            self.h = None
