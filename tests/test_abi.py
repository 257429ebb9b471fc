"""C ABI checks that need no GPU: the library loads, exports every function
include/edb.h declares, and validates arguments before touching a device."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(edb_[A-Za-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_header_declares_functions():
    names = declared_functions()
    assert "edb_qcalc_calQ" in names and "edb_fft3d_fft" in names and "edb_efix_fixsol" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    import __graft_entry__ as g

    b = g._build_module()
    if not os.path.exists(b.LIB):
        b.build()
    lib = C.CDLL(b.LIB)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_and_version():
    from entropydecreaseboltzmann_gb300 import lib

    assert lib.edb_version() >= 100
    assert lib.edb_status_string(0) == b"EDB_OK"
    assert lib.edb_status_string(3) == b"EDB_ECUDA"


@pytest.mark.parametrize("N", [2, 65, -1])
def test_bad_mode_count_is_rejected_before_any_device_work(N):
    import entropydecreaseboltzmann_gb300 as e

    with pytest.raises(e.EdbError) as ei:
        e.QCalculator(N, 0)
    assert ei.value.status == 1  # EDB_EINVAL


def test_bad_index_mode_and_gamma_rejected():
    import entropydecreaseboltzmann_gb300 as e

    with pytest.raises(e.EdbError) as ei:
        e.QCalculator(5, 0, index_mode=7)
    assert ei.value.status == 1
    with pytest.raises(e.EdbError) as ei:
        e.QCalculator(5, 0, gamma=-1.0)
    assert ei.value.status == 1


def test_no_cpu_fallback_without_gpu():
    """Without a GPU the compute entry points fail with EDB_ECUDA."""
    import torch

    import entropydecreaseboltzmann_gb300 as e

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(e.EdbError) as ei:
        e.QCalculator(5, 0)
    assert ei.value.status == 3


def test_python_mirror_has_reference_names():
    import entropydecreaseboltzmann_gb300 as e

    for name in ("genB", "closeFilter", "calQ"):
        assert hasattr(e.QCalculator, name)
    for name in ("fft", "ifft"):
        assert hasattr(e.fft3d, name)
    for name in ("EntropyCal", "setAverage", "FixSol"):
        assert hasattr(e.EntropyFix, name)
    for name in ("FEuler", "CFE", "RK2", "SSP3", "RK4", "DUFORT", "setFixEntropy"):
        assert hasattr(e.BKW3D, name)


def test_ctypes_structs_match_header_layout(tmp_path):
    """Every ctypes mirror of a header struct has the C compiler's size and
    field offsets (compiled here from include/edb.h)."""
    import shutil
    import subprocess

    from entropydecreaseboltzmann_gb300 import _lib

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    mirrors = {"edb_qcalc_desc": _lib.QCalcDesc, "edb_qcalc_info": _lib.QCalcInfo,
               "edb_solver_desc": _lib.SolverDesc, "edb_batch_desc": _lib.BatchDesc,
               "edb_server_desc": _lib.ServerDesc, "edb_request": _lib.Request,
               "edb_request_info": _lib.RequestInfo, "edb_server_stats": _lib.ServerStats}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "edb.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_server_descriptor_validated_before_device_work():
    """edb_server_create rejects bad descriptors with EDB_EINVAL before it
    looks for a GPU."""
    import ctypes as C

    from entropydecreaseboltzmann_gb300 import _lib

    lib = _lib.lib
    for field, value in (("scheme", 99), ("dt", 0.0), ("hbm_budget_bytes", -1.0),
                         ("max_live_per_group", -2)):
        d = _lib.ServerDesc()
        d.hbm_budget_bytes, d.scheme, d.dt = 1e9, 4, 0.01
        setattr(d, field, value)
        h = C.c_void_p()
        assert lib.edb_server_create(C.byref(d), C.byref(h)) == 1, field
