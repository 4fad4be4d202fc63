"""Run the reference's own CUDA kernels (oracle/_ref/ref_kernels.cubin).

TEST INFRASTRUCTURE ONLY.  ``oracle/Makefile`` compiles the five kernels of
odeSolver.cpp:757-1099 unmodified (sm_103a cubin).  This module loads that
cubin through the CUDA driver API, fills its ``__constant__`` level tables
exactly as RK43's initialisation does (odeSolver.cpp:1384-1420) and drives
the kernels with the reference's host sequencing -- smooth(), vcycle(),
multigrid() (odeSolver.cpp:652-755, 1101-1147), restated here with the
reference's hard-coded n_levels = 6 and n_cycles = 32 and launch geometry
(block 32x16).  Device buffers come from torch.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

CUBIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                     "ref_kernels.cubin")
N_LEVELS = 6     # odeSolver.cpp:3
N_CYCLES = 32    # odeSolver.cpp:4

KERNELS = {
    "rbgs0": "_Z11rbgs_kernelILi0EEvPdS0_S0_i",
    "rbgs1": "_Z11rbgs_kernelILi1EEvPdS0_S0_i",
    "residual": "_Z15residual_kernelPdS_S_S_i",
    "restriction": "_Z18restriction_kernelPdS_S_i",
    "prolongate": "_Z17prolongate_kernelPdS_i",
    "delta": "_Z14calcuDelta_devPdS_S_S_i",
}


class DimInfo(C.Structure):          # struct.h:81-87
    _fields_ = [("M", C.c_int), ("N", C.c_int), ("K", C.c_int), ("fin_coa", C.c_int),
                ("DH", C.c_double)]


class Inners(C.Structure):           # struct.h:90-97
    _fields_ = [("istart", C.c_int), ("iend", C.c_int), ("jstart", C.c_int), ("jend", C.c_int),
                ("kstart", C.c_int), ("kend", C.c_int)]


def available() -> bool:
    return os.path.exists(CUBIN)


class RefKernels:
    def __init__(self, ni, nk, dh, mu_equi):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")
        self.torch = torch
        self.cu = C.CDLL("libcuda.so.1")
        self.mod = C.c_void_p()
        data = open(CUBIN, "rb").read()
        self._data = C.create_string_buffer(data, len(data))
        self._chk(self.cu.cuModuleLoadData(C.byref(self.mod), self._data), "cuModuleLoadData")
        self.fn = {}
        for k, name in KERNELS.items():
            f = C.c_void_p()
            self._chk(self.cu.cuModuleGetFunction(C.byref(f), self.mod, name.encode()), name)
            self.fn[k] = f
        # level tables, odeSolver.cpp:1384-1417
        self.dims = (DimInfo * N_LEVELS)()
        self.inn = (Inners * N_LEVELS)()
        n, k, h = nk, ni, dh
        self.dims[0] = DimInfo(1, n, k, 1, h)
        for i in range(N_LEVELS - 1):
            n = (n - 1) // 2 + 1
            k = (k - 1) // 2 + 1
            h *= 2
            self.dims[i + 1] = DimInfo(1, n, k, 2 ** (i + 1), h)
        for i in range(N_LEVELS):
            self.inn[i] = Inners(0, 1, 0, self.dims[i].N, 1, self.dims[i].K - 1)
        self._set_global("dimsinfo_dev", self.dims)
        self._set_global("innersinfo_dev", self.inn)
        dev = lambda n_: torch.zeros(n_, dtype=torch.float64, device="cuda")
        self.mu = torch.from_numpy(np.ascontiguousarray(mu_equi).ravel()).cuda()
        self.res = [dev(self.dims[i].N * self.dims[i].K) for i in range(N_LEVELS - 1)]
        self.res2 = [dev(self.dims[i + 1].N * self.dims[i + 1].K) for i in range(N_LEVELS - 1)]
        self.err2 = [dev(self.dims[i + 1].N * self.dims[i + 1].K) for i in range(N_LEVELS - 1)]
        self.delta = dev(nk * ni)

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"CUDA driver error {rc} in {what}")

    def _set_global(self, name, obj):
        ptr = C.c_uint64()
        size = C.c_size_t()
        self._chk(self.cu.cuModuleGetGlobal_v2(C.byref(ptr), C.byref(size), self.mod, name.encode()),
                  name)
        assert size.value == C.sizeof(obj), (name, size.value, C.sizeof(obj))
        self._chk(self.cu.cuMemcpyHtoD_v2(ptr, C.byref(obj), C.sizeof(obj)), "cuMemcpyHtoD")

    def _launch(self, name, grid, args):
        """args: list of ('p', tensor) / ('i', int)"""
        holders = []
        for kind, v in args:
            holders.append(C.c_uint64(v.data_ptr()) if kind == "p" else C.c_int(v))
        arr = (C.c_void_p * len(holders))(*[C.cast(C.byref(h), C.c_void_p) for h in holders])
        self._chk(self.cu.cuLaunchKernel(self.fn[name], grid[0], grid[1], grid[2], 32, 16, 1, 0,
                                         None, arr, None), name)

    @staticmethod
    def _g(n, b):
        return (n + b - 1) // b

    def _grid(self, level):
        d = self.inn[level]
        return (self._g(d.kend - d.kstart, 32), self._g(d.jend - d.jstart, 16), 1)

    # smooth(), odeSolver.cpp:741-755
    def smooth(self, u, f, level, n=N_CYCLES):
        g = self._grid(level)
        for _ in range(n):
            self._launch("rbgs0", g, [("p", u), ("p", f), ("p", self.mu), ("i", level)])
            self._launch("rbgs1", g, [("p", u), ("p", f), ("p", self.mu), ("i", level)])

    # vcycle(), odeSolver.cpp:1101-1147
    def vcycle(self, u, f, level=0):
        if level >= N_LEVELS - 1:
            self.smooth(u, f, level)
            return
        r, r2, e2 = self.res[level], self.res2[level], self.err2[level]
        self.smooth(u, f, level)
        self._launch("residual", self._grid(level),
                     [("p", r), ("p", u), ("p", f), ("p", self.mu), ("i", level)])
        c = self.dims[level + 1]
        self._launch("restriction", (self._g(c.K - 2, 32), self._g(c.N, 16), 1),
                     [("p", r2), ("p", r), ("p", e2), ("i", level + 1)])
        self.vcycle(e2, r2, level + 1)
        self._launch("prolongate", (self._g(c.K - 1, 32), self._g(c.N - 1, 16), 1),
                     [("p", u), ("p", e2), ("i", level + 1)])
        self.smooth(u, f, level)

    def residual_norm(self, u, f):
        """calcuDelta_dev + cublasDnrm2 (odeSolver.cpp:693-694)."""
        self._launch("delta", self._grid(0),
                     [("p", u), ("p", f), ("p", self.mu), ("p", self.delta), ("i", 0)])
        self.torch.cuda.synchronize()
        return float(self.torch.linalg.vector_norm(self.delta).item())

    # multigrid()'s device loop, odeSolver.cpp:688-705 (capped here)
    def multigrid(self, u, f, eps=1e-9, max_cycles=1000):
        delta = self.residual_norm(u, f)
        it = 0
        while delta > eps and it < max_cycles:
            self.vcycle(u, f, 0)
            delta = self.residual_norm(u, f)
            it += 1
        return it, delta

    def to_dev(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).ravel()).cuda()

    def close(self):
        if self.mod:
            self.torch.cuda.synchronize()
            self.cu.cuModuleUnload(self.mod)
            self.mod = C.c_void_p()
