"""Files around the RK43 run: the reference's initial-displacement input
(odeSolver.cpp:96-128), its snapshot records (:1442-1456, :1638-1652) and
the checkpoint / restart file.  The file formats need no GPU; snapshots and
checkpoints read the device state."""
import numpy as np
import pytest

from qdeqcycle_fdm_gb300 import api, _lib


def test_initial_u_file_layout(tmp_path):
    ni, nk = 7, 5
    rng = np.random.default_rng(0)
    u0 = rng.normal(size=(nk, ni))
    f = tmp_path / "u0.bin"
    u0.tofile(f)                    # ni * nk doubles, column index fastest
    U = api.load_initial_u(f, ni, nk)
    assert U.shape == (nk + 2, ni + 2)
    assert np.array_equal(U[1:-1, 1:-1], u0)
    assert not U[0].any() and not U[-1].any() and not U[:, 0].any() and not U[:, -1].any()
    g = tmp_path / "u1.bin"
    api.save_initial_u(g, U)
    assert f.read_bytes() == g.read_bytes()


def test_initial_u_short_file_is_an_error(tmp_path):
    f = tmp_path / "short.bin"
    np.zeros(10).tofile(f)
    with pytest.raises(_lib.QdError):
        api.load_initial_u(f, 7, 5)
    with pytest.raises(_lib.QdError):
        api.load_initial_u(tmp_path / "missing.bin", 7, 5)


def _sim(n=33):
    from qdeqcycle_fdm_gb300 import config, problem
    cfg = config.small(n)
    prob = problem.build_problem(cfg)
    return prob, cfg


@pytest.mark.gpu
def test_checkpoint_resumes_bit_for_bit(tmp_path):
    import dataclasses
    prob, cfg = _sim(65)
    mg = dataclasses.replace(cfg.mg, precision=1, surface_prolong=1, coarse_solve=1, tol=1e-9)
    a = api.Simulation(prob, mg)
    a.start()
    a.step(15)
    ck = tmp_path / "run.ckp"
    a.solver.checkpoint_save(ck)
    a.step(10)
    sa = a.state()
    a.close()
    b = api.Simulation(prob, mg)
    b.solver.checkpoint_load(ck)
    b.step(10)
    sb = b.state()
    b.close()
    for k in ("Slip", "psi", "V", "Ts", "dpsi", "U"):
        assert np.array_equal(sa[k], sb[k]), k
    assert sa["t"] == sb["t"] and sa["dt"] == sb["dt"] and sa["it"] == sb["it"]


@pytest.mark.gpu
def test_snapshot_records_match_the_state(tmp_path):
    prob, cfg = _sim(33)
    sim = api.Simulation(prob, cfg.mg)
    sim.start()
    sim.step(3)
    st = sim.state()
    nz, nx = prob.nz, prob.nx
    full, per, asy = tmp_path / "f.bin", tmp_path / "p.bin", tmp_path / "a.bin"
    sim.solver.snapshot(full, full=True)
    sim.solver.snapshot(per, full=False)
    sim.solver.snapshot(asy, full=True, asynchronous=True)
    sim.solver.snapshot_wait()
    r = np.fromfile(full)
    assert r.size == 1 + 4 * nz + nx * nz + 3 * nz + 1
    assert r[0] == st["t"] and r[-1] == st["dt"]
    assert np.array_equal(r[1:1 + nz], st["V"])
    assert np.array_equal(r[1 + nz:1 + 2 * nz], st["Slip"])
    assert np.array_equal(r[1 + 2 * nz:1 + 3 * nz], st["Ts"])
    assert np.array_equal(r[1 + 3 * nz:1 + 4 * nz], st["psi"])
    assert np.array_equal(r[1 + 4 * nz:1 + 4 * nz + nx * nz].reshape(nz, nx), st["U"])
    o = 1 + 4 * nz + nx * nz
    assert np.array_equal(r[o + nz:o + 2 * nz], prob.a) and np.array_equal(r[o + 2 * nz:o + 3 * nz], prob.b)
    p = np.fromfile(per)
    assert p.size == 1 + 4 * nz + 1
    assert np.array_equal(p[:1 + 4 * nz], r[:1 + 4 * nz]) and p[-1] == r[-1]
    assert asy.read_bytes() == full.read_bytes()
    sim.close()
