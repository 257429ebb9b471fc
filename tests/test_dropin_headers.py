"""The C++ drop-in headers (entropydecreaseboltzmann_gb300/cpp): the
reference's own drivers compile and link against them unchanged (CPU, when
the reference sources are present), other types are rejected at compile
time, and the repo's reference-style driver builds."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "entropydecreaseboltzmann_gb300", "cpp")
INC = os.path.join(ROOT, "include")
PKG = os.path.join(ROOT, "entropydecreaseboltzmann_gb300")
from oracle.oracle import REF_SRC as REF  # noqa: E402


def gxx():
    cc = shutil.which("g++")
    if not cc:
        pytest.skip("no C++ compiler")
    return cc


def libedb():
    import __graft_entry__ as g

    b = g._build_module()
    if not os.path.exists(b.LIB):
        b.build()
    return b.LIB


def compile_and_link(src, out, extra_inc=()):
    cmd = [gxx(), "-std=c++14", "-O1", *[f"-I{d}" for d in extra_inc], f"-I{CPP}", f"-I{INC}",
           src, f"-L{PKG}", "-ledb", f"-Wl,-rpath,{PKG}", "-o", out]
    return subprocess.run(cmd, capture_output=True, text=True)


@pytest.mark.parametrize("driver", ["test.cpp", "testBKW3D.cpp", "testEntropyFix.cpp",
                                    "testfft.cpp"])
def test_reference_drivers_build_against_dropin_headers(tmp_path, driver):
    """The reference's drivers (and BKW.h) compile unchanged with the drop-in
    QCalculator.h / fft3d.h / EntropyFix.h first on the include path and link
    against libedb.so, with no FFTW."""
    if not os.path.isdir(REF):
        pytest.skip("reference sources not present")
    libedb()
    # the driver and the reference headers it keeps (BKW.h, TimeWatch.h) go
    # to a scratch directory, so its quoted includes find the drop-ins
    for f in (driver, "BKW.h", "TimeWatch.h"):
        shutil.copy(os.path.join(REF, f), tmp_path / f)
    r = compile_and_link(str(tmp_path / driver), str(tmp_path / "a.out"))
    assert r.returncode == 0, r.stderr[-3000:]


def test_dropin_rejects_other_types(tmp_path):
    src = tmp_path / "bad.cpp"
    src.write_text('#include <complex>\n#include "QCalculator.h"\n'
                   "int main() { QCalculator<std::complex<float>, float> q(5, 0); return 0; }\n")
    r = subprocess.run([gxx(), "-std=c++14", f"-I{CPP}", f"-I{INC}", "-fsyntax-only", str(src)],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "complex<double>" in r.stderr


def test_repo_driver_builds(tmp_path):
    libedb()
    r = compile_and_link(os.path.join(ROOT, "tests", "cpp", "dropin_driver.cpp"),
                         str(tmp_path / "drv"))
    assert r.returncode == 0, r.stderr[-3000:]
