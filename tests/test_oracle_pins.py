"""Pin the CPU oracle to the reference's own host functions.

The golden vectors in ``tests/golden/ref_host_golden.npz`` were produced by
the reference's fault.cpp / odeSolver.cpp compiled from source
(``tests/golden/make_golden.py``).  On x86-64 the oracle and the reference
compile to the same IEEE operations (no FMA contraction, same libm), so the
comparison is bit-exact there; elsewhere it allows a few ulps.
"""
import os
import platform

import numpy as np
import pytest

import oracle

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_host_golden.npz"))
EXACT = platform.machine() in ("x86_64", "AMD64")


def same(a, b, rtol=1e-14):
    if EXACT:
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=rtol, atol=0)


@pytest.fixture(scope="module", autouse=True)
def _build(oracle_lib):
    return oracle_lib


def test_eval_stress_on_fault():
    Ts, Tn = oracle.eval_stress_on_fault(int(G["stress_ni"]), int(G["stress_nk"]),
                                         float(G["stress_dh"]), G["stress_U"], G["stress_mu"],
                                         G["stress_Tau_n0"])
    nk = int(G["stress_nk"])
    same(Ts[1:nk + 1], G["stress_Ts"][1:nk + 1])
    same(Tn[1:nk + 1], G["stress_Tn"][1:nk + 1])


def test_nrsearch_matches_reference():
    nk = int(G["nr_nk"])
    V, iters, st = oracle.nrsearch(nk, G["nr_Ts"], G["nr_Tn"], G["nr_a"], G["nr_eta"],
                                   G["nr_psi"], 1e-6, G["nr_seed"])
    assert st == 0
    same(V[1:nk + 1], G["nr_V"][1:nk + 1])
    assert iters[1:nk + 1].max() < 200


def test_cal_dpsi_edges():
    nk = int(G["dp_nk"])
    d = oracle.cal_dpsi(nk, G["dp_psi"], G["dp_b"], G["dp_V"], 0.6, 1e-6, 0.008)
    same(d[1:nk + 1], G["dp_out"][1:nk + 1])
    assert d[5] == 0.0 and d[6] == 0.0 and d[7] == 0.0   # b <= 1e-3, exp overflow


def test_compute_error():
    nk = int(G["err_nk"])
    e = oracle.compute_error(nk, G["err_s3"], G["err_p3"], G["err_s4"], G["err_p4"])
    same(np.array(e), G["err_out"])


def test_compute_step_size():
    for it, dt, tot, e0, e1, val in G["ss_cases"]:
        got = oracle.compute_step_size(int(it), dt, 1e-5, 1e8, tot, 1e-7, [e0, e1])
        same(np.array(got), np.array(val))


def test_set_boundary_and_extend_crew():
    ni, nk = int(G["bc_ni"]), int(G["bc_nk"])
    U = G["bc_U"].copy()
    oracle.set_boundary(ni, nk, U, G["bc_slip"], G["bc_shift"], 1e-9, 3.2e9, 0.62, 1.7e6)
    same(U, G["bc_out"])
    U = G["bc_U"].copy()
    oracle.extend_crew(ni, nk, U)
    same(U, G["ec_out"])


def test_interp_basis_path():
    """SetMedium's interpolants, through the oracle's precomputed-basis path."""
    L = oracle.lib()
    for row in G["interp"]:
        z = np.ascontiguousarray(row[:12])
        xi, yi, want_x, want_z = row[12:]
        same(np.array(L.qo_interp_xedge(oracle._p(z), xi, yi)), np.array(want_x))
        same(np.array(L.qo_interp_zedge(oracle._p(z), xi, yi)), np.array(want_z))


@pytest.mark.skipif(oracle.ref_host() is None, reason="reference sources not built here")
def test_live_nrsearch_against_reference():
    """Fresh random cases straight through the reference's NRsearch."""
    R = oracle.ref_host()
    rng = np.random.default_rng(7)
    nk = 500
    nz = nk + 2
    # keep (Ts)/(a|Tn|) well below 710: past it the reference's first Newton
    # step lands where sinh overflows and its NRsearch exit(0)s the process
    a = np.r_[0, rng.uniform(0.008, 0.03, nk), 0]
    eta = np.r_[0, rng.uniform(1, 8, nk), 0]
    Tn = np.r_[0, -rng.uniform(20, 100, nk), 0]
    psi = np.r_[0, rng.uniform(0.5, 0.9, nk), 0]
    Ts = np.r_[0, rng.uniform(-5, 30, nk), 0]
    V0 = np.zeros(nz)
    Vr = V0.copy()
    R.ref_nrsearch(nk, oracle._p(Ts), oracle._p(Tn), oracle._p(a), oracle._p(eta),
                   oracle._p(psi), 1e-6, oracle._p(Vr))
    Vo, _, st = oracle.nrsearch(nk, Ts, Tn, a, eta, psi, 1e-6, V0)
    assert st == 0
    same(Vo[1:-1], Vr[1:-1])


def test_nrsearch_overflow_reports_instead_of_exiting():
    """A first Newton step past sinh's range gives NaN; the reference prints
    and exit(0)s (fault.cpp:211-225), the oracle reports the node."""
    nk = 3
    z = np.zeros(nk + 2)
    a = z + 0.005
    eta = z + 4.0
    Tn = z - 10.0
    psi = z + 0.7
    Ts = z + 60.0          # fb / fa = 1200 > 710
    V, _, st = oracle.nrsearch(nk, Ts, Tn, a, eta, psi, 1e-6, z)
    assert st == -2        # first failing node is k = 1


def test_set_medium_constant_and_layered():
    """Homogenised face moduli: exact for constant mu; harmonic mean for mu(z)."""
    ni = nk = 17
    nx, nz = ni + 2, nk + 2
    mu = np.full((nz, nx), 30.0)
    _, me = oracle.set_medium(ni, nk, mu)
    W = 2 * nx - 1
    # x-faces on node rows, z-faces between node rows (interior columns)
    xf = me[2:2 * nk + 1:2, 3:2 * ni:2]
    zf = me[1:2 * nk + 2:2, 4:2 * ni - 1:2]
    np.testing.assert_allclose(xf, 30.0, rtol=1e-14)
    np.testing.assert_allclose(zf, 30.0, rtol=1e-14)
    assert me.shape == (2 * nz - 1, W)
