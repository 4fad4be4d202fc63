"""The C++ drop-in surface (include/qdeq_functions.h) exports the reference's
hot-path functions under the reference's own (mangled) names, so code built
against QDEqCycle_FDM's functions.h / struct.h links to this library."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"

DROPIN = ["RK43", "ode_solve", "extend_crew", "setBoundary", "eval_stress_on_fault", "NRsearch",
          "cal_dpsi", "computeError", "computeStepSize", "SetMedium"]


def exported(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True,
                         check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


@pytest.fixture(scope="module")
def syms(gpu_lib):
    from qdeqcycle_fdm_gb300.build import LIB
    return exported(LIB)


def test_dropin_functions_exported(syms):
    names = {s for s in syms if s.startswith("_Z")}
    for fn in DROPIN:
        assert any(f"{len(fn)}{fn}" in s for s in names), fn
    assert "qd_dropin_configure" in syms and "qd_dropin_bind" in syms


def test_struct_layout_matches_reference_sizes(tmp_path):
    """sizeof/offsetof of the kept structs, compiled from our header."""
    src = tmp_path / "s.cpp"
    src.write_text('#include "qdeq_struct.h"\n#include <cstdio>\n#include <cstddef>\n'
                   'int main(){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(PARAMS), sizeof(GRID), '
                   'offsetof(PARAMS, totTol), offsetof(GRID, i0), sizeof(RATE_STATE_LAW), '
                   'sizeof(FAULT));}\n')
    exe = tmp_path / "s"
    subprocess.run(["g++", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    ours = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    if not os.path.isdir(REF):
        assert ours[0] != "0"
        return
    src2 = tmp_path / "r.cpp"
    src2.write_text(f'#include "{REF}/struct.h"\n#include <cstdio>\n#include <cstddef>\n'
                    'int main(){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(PARAMS), sizeof(GRID), '
                    'offsetof(PARAMS, totTol), offsetof(GRID, i0), sizeof(RATE_STATE_LAW), '
                    'sizeof(FAULT));}\n')
    exe2 = tmp_path / "r"
    subprocess.run(["g++", str(src2), "-o", str(exe2)], check=True)
    ref = subprocess.run([str(exe2)], capture_output=True, text=True, check=True).stdout.split()
    assert ours == ref


@pytest.mark.skipif(not os.path.isdir(REF) or shutil.which("g++") is None,
                    reason="reference sources not present")
def test_reference_main_links_against_dropin(syms, tmp_path):
    """The reference's own main (eq_cycle.cpp) needs RK43 / extend_crew /
    SetMedium with exactly the mangled names this library exports."""
    obj = tmp_path / "eq_cycle.o"
    subprocess.run(["g++", "-c", "-std=c++11", "-include", os.path.join(ROOT, "oracle", "ref_shim.h"),
                    os.path.join(REF, "eq_cycle.cpp"), "-o", str(obj)], check=True)
    undef = subprocess.run(["nm", "-u", str(obj)], capture_output=True, text=True,
                           check=True).stdout.split()
    needed = [s for s in undef if any(f"{len(f)}{f}" in s for f in ("RK43", "extend_crew", "SetMedium"))]
    assert len(needed) == 3
    for s in needed:
        assert s in syms, s
