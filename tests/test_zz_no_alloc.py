"""qd_residual_norm_noalloc: the residual norm for callers that cannot
allocate device memory (a host framework that owns all device memory, or
code where a cudaMalloc would synchronise the device mid-stream).

The entry point gets the caller's own device arrays and keeps its block
partial sums in a static device array; it must give the same norm as the
solver's qd_mg_residual_norm on the same field, call after call.  This file
is collected last so that a failure here does not hide the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from qdeqcycle_fdm_gb300 import _lib, api, config, problem

pytestmark = pytest.mark.gpu


def level0_faces(prob, P):
    """The solver's level-0 face moduli, built from mu_equi on the host."""
    me = prob.mu_equi
    N, K = prob.nk, prob.ni
    cx = np.zeros((N, P))
    cz = np.zeros((N + 1, P))
    for j in range(N):
        cx[j, :K - 1] = me[(j + 1) * 2, 3:2 * K:2]
    for j in range(N + 1):
        cz[j, :K] = me[2 * j + 1, 2:2 * K + 2:2]
    return cx, cz


def test_noalloc_norm_matches_solver_norm(gpu_lib):
    import torch
    cfg = config.small(129, mu_profile="layered", layer_depth_km=20.0)
    prob = problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])
    rng = np.random.default_rng(11)
    U = np.zeros((prob.nz, prob.nx))
    U[1:-1, 1:-1] = rng.normal(size=(prob.nk, prob.ni))
    s = api.Solver(prob.ni, prob.nk, prob.dh, prob.mu_equi, prob.mu_node, cfg.mg)
    s.upload_u(U)
    want = s.residual_norm()

    N, K = prob.nk, prob.ni
    P = (K + 31) // 32 * 32
    cx, cz = level0_faces(prob, P)
    u = np.zeros((N, P))
    u[:, :K] = U[1:-1, 1:-1]
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (u, cx, cz)]
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    L = _lib.load()
    got = []
    for _ in range(2):      # the static scratch keeps the last call's contents
        out = C.c_double(-1.0)
        rc = L.qd_residual_norm_noalloc(dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), N, K,
                                        P, prob.dh, C.c_void_p(stream.cuda_stream), C.byref(out))
        assert rc == 0, L.qd_last_error()
        got.append(out.value)
    for g in got:
        assert abs(g - want) <= 1e-12 * want, (g, want)
    assert got[0] == got[1]


def test_noalloc_rejects_grids_beyond_its_scratch(gpu_lib):
    L = _lib.load()
    out = C.c_double(0.0)
    dummy = C.c_void_p(8)      # never dereferenced: the size check comes first
    # too many rows and columns; and a grid whose block count would fit but
    # whose columns exceed 4097
    for nk, ni, pitch in ((8193, 8193, 8224), (4097, 4300, 4320), (5000, 129, 160)):
        rc = L.qd_residual_norm_noalloc(dummy, dummy, dummy, nk, ni, pitch, 1.0, None, C.byref(out))
        assert rc == _lib.QD_ERR_ARG, (nk, ni)
        assert b"4097" in L.qd_last_error()
