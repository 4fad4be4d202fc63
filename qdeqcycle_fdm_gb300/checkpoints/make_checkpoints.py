"""Write the named mid-cycle checkpoints of config 1 (1025^2) on the GPU.

Run:  python -m qdeqcycle_fdm_gb300.checkpoints.make_checkpoints

From the steady-sliding start (V = Vp) the cycle settles after its first
rupture into a regular one of about 49.7 simulated years with about 1,900
accepted steps, most of them inside the rupture (dt ~ 1e-2 s).  The run
uses the mixed-precision solver with the solution-history guess (relative
residual 1e-9) and saves:

  config1_1025_rupture3       the 100th accepted step after the third
                              rupture's onset (max V first above 0.1 m/s):
                              the rupture's plateau of dt ~ 1.6e-2 s, where
                              most of a cycle's steps are taken
  config1_1025_interseismic3  the first accepted step 10 simulated years
                              after the third rupture's onset: the loading
                              phase, dt ~ 1e7 s, about 40 years before the
                              next rupture

The GPU run is deterministic, so the files are reproducible bit for bit on
the same library build.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from qdeqcycle_fdm_gb300 import api, build, checkpoints, config, problem  # noqa: E402

YEAR_S = config.YEAR_S
ONSET_V = 0.1          # m/s: a rupture's onset
PLATEAU_STEPS = 100    # accepted steps after the onset: inside the rupture's plateau
LOADING_YEARS = 10.0   # simulated years after the onset: the loading phase


def main():
    build.build()
    cfg = config.config1()
    prob = problem.build_problem(cfg)
    mg = config.MGConfig(**{**cfg.mg.__dict__, "precision": 1, "surface_prolong": 1, "coarse_solve": 1})
    sim = api.Simulation(prob, mg)
    sim.solver.set_solution_history(4)
    sim.start()
    k = slice(1, prob.nk + 1)
    onsets, above = [], False
    wrote = {}
    meta0 = {"config": cfg.name, "ni": prob.ni, "nk": prob.nk, "seed": cfg.seed,
             "written_by": "mixed precision, solution-history guess (4), rel 1e-9, V(2,2), 8 levels, "
                           "surface-row prolongation, exact coarsest solve, from steady sliding"}
    while len(wrote) < 2:
        sim.step(1)
        st = sim.solver.rk43_state()
        vmax = float(np.max(st["V"][k]))
        if vmax > ONSET_V and not above:
            onsets.append((st["it"], st["t"]))
        above = vmax > ONSET_V
        if len(onsets) >= 3:
            it3, t3 = onsets[2]
            name = None
            if "rupture3" not in wrote and st["it"] == it3 + PLATEAU_STEPS:
                name = "config1_1025_rupture3"
            elif "interseismic3" not in wrote and st["t"] >= t3 + LOADING_YEARS * YEAR_S:
                name = "config1_1025_interseismic3"
            if name:
                meta = {**meta0, "name": name, "t_years": st["t"] / YEAR_S, "step": st["it"],
                        "max_V": vmax, "dt_s": st["dt"], "rupture_onsets_years": [t / YEAR_S for _, t in onsets]}
                checkpoints.save(checkpoints.path(name), checkpoints.from_state(st), meta)
                wrote[name.split("_")[-1]] = meta
                print(json.dumps(meta), flush=True)
        if st["t"] > 400 * YEAR_S:
            raise RuntimeError("no third rupture within 400 simulated years")
    sim.close()


if __name__ == "__main__":
    main()
