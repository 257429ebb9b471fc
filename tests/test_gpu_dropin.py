"""The repo's reference-style C++ driver (tests/cpp/dropin_driver.cpp), built
against the drop-in headers and libedb.so, run on the GPU: calQ equals the
reference's golden output (relative L2 <= 1e-12), fft/ifft match numpy
(<= 1e-13), EntropyCal / FixSol / funF / filtering match the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "entropydecreaseboltzmann_gb300", "cpp")
INC = os.path.join(ROOT, "include")
PKG = os.path.join(ROOT, "entropydecreaseboltzmann_gb300")


@pytest.mark.parametrize("N,alpha,filt", [(5, 0, 1), (8, 1, 0)])
def test_cpp_dropin_driver(tmp_path, golden, oracle, N, alpha, filt):
    import __graft_entry__ as g

    b = g._build_module()
    if not os.path.exists(b.LIB):
        b.build()
    cc = shutil.which("g++")
    if not cc:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "drv"
    r = subprocess.run([cc, "-std=c++14", "-O1", f"-I{CPP}", f"-I{INC}",
                        os.path.join(ROOT, "tests", "cpp", "dropin_driver.cpp"), f"-L{PKG}", "-ledb",
                        f"-Wl,-rpath,{PKG}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    tag = f"N{N}_a{alpha}_f{filt}"
    fin = golden[f"calq_in_{tag}"].astype(np.complex128)
    NQ = N ** 3
    f = 0.2 + np.random.default_rng(N).uniform(0.0, 1.0, NQ)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as fh:
        np.array([N, alpha, filt], dtype=np.int32).tofile(fh)
        fin.tofile(fh)
        f.tofile(fh)
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    raw = np.fromfile(out, dtype=np.float64)
    Q = raw[:2 * NQ].view(np.complex128)
    back = raw[2 * NQ:4 * NQ].view(np.complex128)
    Fh = raw[4 * NQ:6 * NQ].view(np.complex128)
    H = raw[6 * NQ]
    f_fixed = raw[6 * NQ + 1:7 * NQ + 1]
    funF, filt1 = raw[7 * NQ + 1:7 * NQ + 3]
    want = golden[f"calq_out_{tag}"]
    assert np.linalg.norm(Q - want) / np.linalg.norm(want) <= 1e-12
    ref_fft = np.fft.fftn(fin.reshape(N, N, N)).reshape(-1)
    assert np.max(np.abs(Fh - ref_fft)) <= 1e-13 * np.max(np.abs(ref_fft))
    assert np.max(np.abs(back - fin)) <= 1e-13 * np.max(np.abs(fin))
    from oracle.oracle import EntropyFixOracle

    eo = EntropyFixOracle(oracle, NQ)
    H_o = eo.EntropyCal(f)
    assert abs(H - H_o) <= 1e-12 * abs(H_o)
    g_o = f.copy()
    eo.FixSol(g_o, H_o - 1e-3)
    assert np.max(np.abs(f_fixed - g_o)) <= 1e-9 * np.max(np.abs(g_o))
    assert "Averafe f" in r.stdout
    assert abs(funF - oracle.funF(alpha, 0.7, 1.3)) <= 1e-14
    assert abs(filt1 - oracle.filtering(N, 1)) <= 1e-14
