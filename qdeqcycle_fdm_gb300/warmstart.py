"""The learned warm start (``include/qdeq_unet.h``): a BF16 U-Net that
predicts the change a stage solve makes to u, trained online on the
multigrid's own solutions with the library's tensor-core kernels.

Host arrays follow the header: inputs ``x`` are float32 [5, nk, ni],
targets and outputs float32 [nk, ni], parameters a flat float32 vector.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, load

MODE_OFF, MODE_TRAIN, MODE_PREDICT = 0, 1, 2


def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class UNet:
    def __init__(self, nk: int, ni: int, seed: int = 1):
        self.L = load()
        self.nk, self.ni = nk, ni
        h = C.c_void_p()
        check(self.L.qd_unet_create(nk, ni, seed, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.L.qd_unet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        return int(self.L.qd_unet_num_params(self.h))

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        check(self.L.qd_unet_get_params(self.h, _f(out)))
        return out

    def set_params(self, theta) -> None:
        t = np.ascontiguousarray(theta, dtype=np.float32)
        assert t.size == self.num_params
        check(self.L.qd_unet_set_params(self.h, _f(t)))

    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((self.nk, self.ni), dtype=np.float32)
        check(self.L.qd_unet_forward_host(self.h, _f(x), _f(y)))
        return y

    def loss_grad(self, x, target):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        loss = C.c_float(0)
        g = np.empty(self.num_params, dtype=np.float32)
        check(self.L.qd_unet_loss_grad_host(self.h, _f(x), _f(t), C.byref(loss), _f(g)))
        return float(loss.value), g

    def train_step(self, x, target, lr: float = 1e-3) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        loss = C.c_float(0)
        check(self.L.qd_unet_train_step_host(self.h, _f(x), _f(t), lr, C.byref(loss)))
        return float(loss.value)

    def attach(self, solver, mode: int, lr: float = 1e-3) -> None:
        """Couple to an ``api.Solver`` of the same grid (MODE_TRAIN,
        MODE_PREDICT or MODE_OFF)."""
        check(self.L.qd_solver_warm_start(solver.h, self.h if mode else None, mode, lr))

    @staticmethod
    def set_gate(solver, ratio: float) -> None:
        """Prediction mode's gate: the network corrects a solve's guess only
        when the guess's residual exceeds ratio x the solve's threshold;
        ratio 0 (the default): when the guess would need more than 1 + cost
        V-cycles at the solver's measured reduction per cycle (set_cost,
        default 2)."""
        check(solver.L.qd_solver_warm_start_gate(solver.h, float(ratio)))

    @staticmethod
    def set_cost(solver, cycles: float) -> None:
        """The measured gate's cost of one correction in V-cycles (default
        2): the network runs where a guess needs more than 1 + cost cycles."""
        check(solver.L.qd_solver_warm_start_cost(solver.h, float(cycles)))

    def time(self, what: str = "forward", reps: int = 10):
        """(microseconds per run, tensor-core FLOPs per run) of one inference
        ("forward"), one training step without the update ("train") or the
        first, full-grid 16 -> 16 channel convolution alone ("conv16")."""
        us, fl = C.c_double(0), C.c_double(0)
        code = {"forward": 0, "train": 1, "conv16": 2}[what]
        check(self.L.qd_unet_time(self.h, code, reps, C.byref(us), C.byref(fl)))
        return us.value, fl.value

    def stats(self):
        n = C.c_longlong(0)
        loss = C.c_float(0)
        check(self.L.qd_unet_stats(self.h, C.byref(n), C.byref(loss)))
        return int(n.value), float(loss.value)


def _main():
    """python -m qdeqcycle_fdm_gb300.warmstart [n] [reps]: time one inference
    and one training step of a freshly initialised network on an n x n grid
    (random input and target)."""
    import sys
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 1025
    reps = int(sys.argv[2]) if len(sys.argv) > 2 else 10
    rng = np.random.default_rng(0)
    net = UNet(n, n, seed=1)
    theta = net.get_params()
    net.set_params(theta + 0.01 * rng.standard_normal(theta.size).astype(np.float32))
    x = rng.standard_normal((5, n, n)).astype(np.float32)
    t = rng.standard_normal((n, n)).astype(np.float32)
    net.loss_grad(x, t)                       # uploads input and target
    for what in ("forward", "train"):
        us, fl = net.time(what, reps)
        print(f"{what}: {us:.1f} us, {fl / 1e9:.1f} GFLOP, {fl / (us * 1e-6) / 1e12:.1f} TFLOP/s")
    net.close()


if __name__ == "__main__":
    _main()
