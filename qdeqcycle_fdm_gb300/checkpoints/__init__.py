"""Fault-state checkpoints of the earthquake cycle: named mid-cycle states
that every measurement of a workload starts from.

An accepted RK43 step leaves behind only Slip, psi, t, dt, the error
history errA and the step count (odeSolver.cpp:1605-1636): the displacement
u is the elliptic solution for Slip at t, and V, dpsi follow from u, psi by
the stress, Newton and aging-law updates.  So a checkpoint holds those
(a few tens of KB at 1025^2) and a run restarts from it with the commit's
refresh solve (``api.Simulation.resume`` on the GPU, the oracle's
``Simulation.resume`` on the host): every arm of a measurement then times
the same accepted steps from the same state.

The files are written by ``make_checkpoints.py`` beside this module, which
runs the cycle from the steady-sliding start on the GPU and saves states at
named points of a later cycle.
"""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
KEYS = ("Slip", "psi", "t", "dt", "errA0", "errA1", "it")


def path(name: str) -> str:
    return os.path.join(HERE, f"{name}.npz")


def save(fname: str, state: dict, meta: dict) -> None:
    """state: Slip, psi (nz arrays) and the scalars t, dt, errA0, errA1, it."""
    np.savez_compressed(fname, Slip=np.asarray(state["Slip"], dtype=np.float64),
                        psi=np.asarray(state["psi"], dtype=np.float64),
                        scalars=np.array([state["t"], state["dt"], state["errA0"], state["errA1"]]),
                        it=np.array([int(state["it"])], dtype=np.int64),
                        meta=np.array(json.dumps(meta)))


def load(name_or_path: str) -> dict:
    """The checkpoint as a dict with KEYS and 'meta' (a dict)."""
    p = name_or_path if name_or_path.endswith(".npz") else path(name_or_path)
    with np.load(p) as z:
        sc = z["scalars"]
        return {"Slip": z["Slip"].copy(), "psi": z["psi"].copy(), "t": float(sc[0]), "dt": float(sc[1]),
                "errA0": float(sc[2]), "errA1": float(sc[3]), "it": int(z["it"][0]),
                "meta": json.loads(str(z["meta"]))}


def from_state(st: dict) -> dict:
    """A checkpoint dict from a solver's rk43_state() (or the oracle's state())."""
    return {"Slip": st["Slip"].copy(), "psi": st["psi"].copy(), "t": float(st["t"]), "dt": float(st["dt"]),
            "errA0": float(st["errA"][0]), "errA1": float(st["errA"][1]), "it": int(st["it"])}
