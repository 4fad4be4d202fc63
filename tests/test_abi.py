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


def struct_fields(header, name):
    """(C type, field name) pairs of `typedef struct name { ... } name;`."""
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, flags=re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        m = re.match(r"((?:unsigned |const )*(?:long long|int|double|float|char)\s*\**)\s*(.*)", decl)
        ctype, names = m.group(1).strip(), m.group(2)
        for n in names.split(","):
            out.append((ctype, n.strip()))
    return out


@pytest.mark.parametrize("cname, pyname", [("qd_mg_options", "MgOptions"), ("qd_rk43_params", "Rk43Params"),
                                           ("qd_stats", "Stats"), ("qd_tuning", "Tuning")])
def test_ctypes_structs_follow_the_header(cname, pyname):
    """The Python mirrors of the C-ABI structs hold the header's fields in
    its order with types of the same size (a field added on one side only
    would shift every field after it)."""
    import ctypes as C
    from qdeqcycle_fdm_gb300 import _lib
    sizes = {"int": C.sizeof(C.c_int), "long long": C.sizeof(C.c_longlong), "double": C.sizeof(C.c_double),
             "float": C.sizeof(C.c_float), "char": 1, "unsigned int": C.sizeof(C.c_uint)}
    header = struct_fields("qdeq.h", cname)
    py = getattr(_lib, pyname)._fields_
    assert [n for _, n in header] == [n for n, _ in py]
    for (ctype, n), (_, pytype) in zip(header, py):
        assert sizes[ctype] == C.sizeof(pytype), (n, ctype, pytype)
