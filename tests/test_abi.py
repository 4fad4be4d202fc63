"""The C-ABI library builds for sm_103a here, loads without a GPU, and
exports every entry point include/qdeq.h and include/qdeq_unet.h declare."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qd_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(gpu_lib):
    names = declared("qdeq.h")
    assert len(names) >= 20
    names += declared("qdeq_unet.h")
    missing = [n for n in names if not hasattr(gpu_lib, n)]
    assert not missing, missing


def test_python_bindings_cover_header():
    from qdeqcycle_fdm_gb300 import _lib
    bound = {n for n, _, _ in _lib.EXPORTS}
    assert set(declared("qdeq.h")) <= bound
    assert set(declared("qdeq_unet.h")) <= bound


def test_version_and_defaults(gpu_lib):
    from qdeqcycle_fdm_gb300._lib import MgOptions
    assert b"sm_103a" in gpu_lib.qd_version()
    o = MgOptions()
    import ctypes
    gpu_lib.qd_default_options(ctypes.byref(o))
    assert (o.n_levels, o.nu_pre, o.nu_post, o.nu_coarse, o.tol_mode, o.tol) == (6, 32, 32, 32, 0, 1e-9)


def test_bad_arguments_are_rejected_without_gpu(gpu_lib):
    import ctypes
    from qdeqcycle_fdm_gb300._lib import MgOptions, QD_ERR_ARG
    o = MgOptions()
    gpu_lib.qd_default_options(ctypes.byref(o))
    h = ctypes.c_void_p()
    assert gpu_lib.qd_solver_create(1, 1, 1.0, None, None, ctypes.byref(o), ctypes.byref(h)) == QD_ERR_ARG
    assert gpu_lib.qd_last_error()
