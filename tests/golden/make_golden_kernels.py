"""Golden vectors from the reference's own CUDA kernels (run on a GPU).

Loads oracle/_ref/ref_kernels.cubin (the reference's odeSolver.cpp kernels,
compiled unmodified by oracle/Makefile) through oracle/refkernels.py, drives
them with the reference's host sequencing on a seeded 65 x 65 problem and
writes ref_kernels_golden.npz (to the path given, default next to this
script): one smooth() at level 0, one coarse-level smooth() with a non-zero
right-hand side, one residual/restriction/prolongation, one V-cycle and a
full multigrid() solve to the reference's absolute 1e-9.

    python tests/golden/make_golden_kernels.py [out.npz]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import refkernels  # noqa: E402
from qdeqcycle_fdm_gb300 import config, problem  # noqa: E402


def inputs():
    cfg = config.small(65, mu_profile="layered", layer_depth_km=20.0)
    prob = problem.build_problem(cfg, homogenize=lambda ni, nk, mu: oracle.set_medium(ni, nk, mu)[1])
    rng = np.random.default_rng(424242)
    u = rng.normal(size=(prob.nk, prob.ni)) * 1e-3
    u[:, 0] = rng.normal(size=prob.nk)
    u[:, -1] = rng.normal(size=prob.nk)
    return prob, u


def main(out):
    oracle.build(ref=False)
    prob, u0 = inputs()
    R = refkernels.RefKernels(prob.ni, prob.nk, prob.dh, prob.mu_equi)
    T = R.torch
    res = {"ni": prob.ni, "nk": prob.nk, "dh": prob.dh, "mu_equi": prob.mu_equi, "u0": u0}
    # level-0 smooth (32 red/black sweeps)
    u = R.to_dev(u0)
    f = T.zeros_like(u)
    R.smooth(u, f, 0)
    res["smooth0"] = u.cpu().numpy().reshape(u0.shape)
    # coarse smooth on level 2 with a random rhs
    d2 = R.dims[2]
    rng = np.random.default_rng(7)
    e_in = rng.normal(size=(d2.N, d2.K)) * 1e-4
    e_in[:, 0] = 0.0                 # the error's Dirichlet columns stay zero
    e_in[:, -1] = 0.0
    e = R.to_dev(e_in)
    fr = R.to_dev(rng.normal(size=(d2.N, d2.K)) * 1e-6)
    res["c_e_in"] = e_in
    res["c_f"] = fr.cpu().numpy().reshape(d2.N, d2.K)
    R.smooth(e, fr, 2)
    res["c_smooth2"] = e.cpu().numpy().reshape(d2.N, d2.K)
    # one V-cycle from u0
    u = R.to_dev(u0)
    R.vcycle(u, f, 0)
    res["vcycle"] = u.cpu().numpy().reshape(u0.shape)
    # multigrid to the reference's absolute tolerance
    u = R.to_dev(u0)
    it, delta = R.multigrid(u, f, 1e-9)
    res["mg_u"] = u.cpu().numpy().reshape(u0.shape)
    res["mg_cycles"] = it
    res["mg_norm"] = delta
    R.close()
    np.savez_compressed(out, **res)
    print("wrote", out, "cycles", it, "norm", delta)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "ref_kernels_golden.npz"))
