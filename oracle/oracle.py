"""ctypes loader for the CPU oracle — TEST INFRASTRUCTURE ONLY.

Two libraries live under ``oracle/``:

* ``_build/libedb_oracle.so`` — the C restatement (``edb_oracle.c``) of the
  reference's QCalculator / fft3d / EntropyFix / BKW3D algorithms.  Built on
  every host by ``make -C oracle``.
* ``_ref/libedbref.so`` — the reference headers themselves compiled unmodified
  (``ref_wrap.cpp``); exists only where the reference sources exist.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  Complex arrays are numpy complex128 of N^3
entries in FFTW order (row-major, last axis fastest).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libedb_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libedbref.so")
# Where the reference's sources are read from: the EDB_REFERENCE_DIR
# environment variable (the reference repository's root), by default the
# read-only copy this build was made against.  Only the build of the compiled
# reference (`make ref`) and the tests that compile the reference's drivers
# read it; nothing on a GPU host does.
REF_ROOT = os.environ.get("EDB_REFERENCE_DIR", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "CalQ")


def reference_sources_present() -> bool:
    """True where the reference's CalQ sources can be read."""
    return os.path.isfile(os.path.join(REF_SRC, "QCalculator.h"))


INDEX_REFERENCE = 0
INDEX_ALIASED = 1
R_REFERENCE = 6.62132
SCHEMES = {"FE": 0, "CFE": 1, "RK2": 2, "SSP3": 3, "RK4": 4, "DUFORT": 5}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def build_oracle(ref: bool = False) -> None:
    """Compile the restatement (and, if ``ref``, the reference) with make."""
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE, f"REF_SRC={REF_SRC}"] + targets, check=True)


class Oracle:
    """The C restatement (``edb_oracle.c``)."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        L = C.CDLL(path)
        self.L = L
        L.edbo_filtering.restype = C.c_double
        L.edbo_filtering.argtypes = [C.c_int, C.c_int]
        L.edbo_funF.restype = C.c_double
        L.edbo_funF.argtypes = [C.c_int, C.c_double, C.c_double]
        L.edbo_funF_quad.restype = C.c_double
        L.edbo_funF_quad.argtypes = [C.c_double, C.c_double, C.c_double]
        L.edbo_lambda.restype = C.c_double
        L.edbo_rval.restype = C.c_double
        L.edbo_rval.argtypes = [C.c_int, C.c_double, C.c_double]
        L.edbo_amax.restype = C.c_int
        L.edbo_amax.argtypes = [C.c_int]
        L.edbo_genB.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, _dp]
        L.edbo_calQ.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
        L.edbo_direct.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, _dp, _dp]
        L.edbo_direct_modes.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, _dp, C.c_int,
                                        C.POINTER(C.c_long), _dp]
        L.edbo_calQ_batch_mt.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _dp, _dp, C.c_int]
        L.edbo_terms.restype = C.c_long
        L.edbo_terms.argtypes = [C.c_int, C.c_int]
        L.edbo_fft3d.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int]
        L.edbo_calentropy.restype = C.c_double
        L.edbo_calentropy.argtypes = [C.c_int, C.c_double, _dp]
        L.edbo_moments.argtypes = [C.c_int, C.c_double, _dp, _dp]
        L.edbo_initial_sinusoid.argtypes = [C.c_int, C.c_double, _dp]
        L.edbo_initial_bkw.argtypes = [C.c_int, C.c_double, C.c_double, _dp]
        L.edbo_bkw_f.restype = C.c_double
        L.edbo_bkw_f.argtypes = [C.c_double, C.c_double]
        L.edbo_bkw_dfds.restype = C.c_double
        L.edbo_bkw_dfds.argtypes = [C.c_double, C.c_double]
        L.edbo_run.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double,
                               C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                               _dp, _dp, _dp, _dp, _dp, C.c_int, _ip]

    # ---- kernel table and collision sum
    def filtering(self, N, beta):
        return self.L.edbo_filtering(N, beta)

    def funF(self, alpha, xi, eta):
        return self.L.edbo_funF(alpha, xi, eta)

    def funF_quad(self, gamma, xi, eta):
        return self.L.edbo_funF_quad(gamma, xi, eta)

    def rval(self, N, gamma=0.0, R=R_REFERENCE):
        return self.L.edbo_rval(N, gamma, R)

    def genB(self, N, gamma=0.0, R=R_REFERENCE, filter=True, mode=INDEX_REFERENCE):
        nq = N ** 3
        B = np.empty(nq * nq, dtype=np.float64)
        rc = self.L.edbo_genB(N, float(gamma), float(R), int(bool(filter)), int(mode), _ptr(B))
        assert rc == 0
        return B

    def calQ(self, N, B, fin, mode=INDEX_REFERENCE):
        fin = np.ascontiguousarray(fin, dtype=np.complex128).reshape(-1)
        out = np.empty_like(fin)
        rc = self.L.edbo_calQ(N, int(mode), _ptr(B), _ptr(fin.view(np.float64)),
                              _ptr(out.view(np.float64)))
        assert rc == 0
        return out

    def calQ_batch(self, N, B, fins, mode=INDEX_REFERENCE, nthreads=None):
        fins = np.ascontiguousarray(fins, dtype=np.complex128)
        S = fins.shape[0]
        out = np.empty_like(fins)
        nthreads = nthreads or os.cpu_count() or 1
        rc = self.L.edbo_calQ_batch_mt(N, int(mode), _ptr(B), S, _ptr(fins.view(np.float64)),
                                       _ptr(out.view(np.float64)), int(nthreads))
        assert rc == 0
        return out

    def direct(self, N, fin, gamma=0.0, R=R_REFERENCE, filter=True):
        fin = np.ascontiguousarray(fin, dtype=np.complex128).reshape(-1)
        out = np.empty_like(fin)
        rc = self.L.edbo_direct(N, float(gamma), float(R), int(bool(filter)),
                                _ptr(fin.view(np.float64)), _ptr(out.view(np.float64)))
        assert rc == 0
        return out

    def direct_modes(self, N, fin, kidx, gamma=0.0, R=R_REFERENCE, filter=True):
        """Direct aliased evaluation at the FFTW flat indices kidx (O(len(kidx) N^3))."""
        fin = np.ascontiguousarray(fin, dtype=np.complex128).reshape(-1)
        k = np.ascontiguousarray(kidx, dtype=np.int64)
        out = np.empty(k.size, dtype=np.complex128)
        rc = self.L.edbo_direct_modes(N, float(gamma), float(R), int(bool(filter)),
                                      _ptr(fin.view(np.float64)), k.size,
                                      k.ctypes.data_as(C.POINTER(C.c_long)),
                                      _ptr(out.view(np.float64)))
        assert rc == 0
        return out

    def terms(self, N, mode):
        return self.L.edbo_terms(N, mode)

    # ---- transforms, entropy, moments
    def fft3d(self, N, x, inverse=False):
        x = np.ascontiguousarray(x, dtype=np.complex128).reshape(-1)
        out = np.empty_like(x)
        self.L.edbo_fft3d(N, N, N, _ptr(x.view(np.float64)), _ptr(out.view(np.float64)),
                          int(bool(inverse)))
        return out

    def calentropy(self, N, R, F):
        F = np.ascontiguousarray(F, dtype=np.complex128).reshape(-1)
        return self.L.edbo_calentropy(N, R, _ptr(F.view(np.float64)))

    def moments(self, N, R, F):
        F = np.ascontiguousarray(F, dtype=np.complex128).reshape(-1)
        out = np.empty(5)
        self.L.edbo_moments(N, R, _ptr(F.view(np.float64)), _ptr(out))
        return out

    def initial_sinusoid(self, N, R):
        F = np.empty(N ** 3, dtype=np.complex128)
        self.L.edbo_initial_sinusoid(N, R, _ptr(F.view(np.float64)))
        return F

    def initial_bkw(self, N, R, s):
        F = np.empty(N ** 3, dtype=np.complex128)
        self.L.edbo_initial_bkw(N, R, s, _ptr(F.view(np.float64)))
        return F

    def bkw_f(self, s, v2):
        return self.L.edbo_bkw_f(s, v2)

    def bkw_dfds(self, s, v2):
        return self.L.edbo_bkw_dfds(s, v2)

    def run(self, N, R, scheme, T0, TEnd, dt, beta=1.0, fix=True, F0=None,
            mode=INDEX_REFERENCE, gamma=0.0, Rb=R_REFERENCE, filter=True, cap=100000):
        nq = N ** 3
        Fhat = np.empty(nq, dtype=np.complex128)
        F = np.empty(nq, dtype=np.complex128)
        raw = np.empty(cap)
        fixed = np.empty(cap)
        ns = C.c_int(0)
        f0p = None
        if F0 is not None:
            F0 = np.ascontiguousarray(F0, dtype=np.complex128).reshape(-1)
            f0p = _ptr(F0.view(np.float64))
        sch = SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        rc = self.L.edbo_run(N, R, sch, int(mode), float(gamma), float(Rb), int(bool(filter)),
                             T0, TEnd, dt, beta, int(bool(fix)), f0p,
                             _ptr(Fhat.view(np.float64)), _ptr(F.view(np.float64)),
                             _ptr(raw), _ptr(fixed), cap, C.byref(ns))
        assert rc == 0
        k = min(ns.value, cap)
        return Fhat, F, raw[:k].copy(), fixed[:k].copy()


class EntropyFixOracle:
    """EntropyFix restated (EntropyFix.h:13-253) on top of ``edbo_efix``."""

    class _S(C.Structure):
        _fields_ = [("Nt", C.c_int), ("eps", C.c_double), ("avg", C.c_double),
                    ("avg_flag", C.c_int)]

    def __init__(self, oracle: Oracle, Nt, eps=1.0e-10):
        self.L = oracle.L
        self.s = self._S()
        self.L.edbo_efix_init.argtypes = [C.POINTER(self._S), C.c_int, C.c_double]
        self.L.edbo_efix_setaverage.argtypes = [C.POINTER(self._S), C.c_int, _dp]
        self.L.edbo_efix_entropy.argtypes = [C.POINTER(self._S), C.c_int, _dp]
        self.L.edbo_efix_entropy.restype = C.c_double
        self.L.edbo_efix_fixsol.argtypes = [C.POINTER(self._S), C.c_int, _dp, C.c_double]
        self.L.edbo_efix_init(C.byref(self.s), int(Nt), float(eps))

    @property
    def average(self):
        return self.s.avg

    def setAverage(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        self.L.edbo_efix_setaverage(C.byref(self.s), f.size, _ptr(f))

    def EntropyCal(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        return self.L.edbo_efix_entropy(C.byref(self.s), f.size, _ptr(f))

    def FixSol(self, f, aim):
        assert f.dtype == np.float64 and f.flags["C_CONTIGUOUS"]
        self.L.edbo_efix_fixsol(C.byref(self.s), f.size, _ptr(f), float(aim))


class Reference:
    """The reference headers compiled unmodified (``ref_wrap.cpp``)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        self.L = L
        L.edbref_qcalc_new.restype = C.c_void_p
        L.edbref_qcalc_new.argtypes = [C.c_int, C.c_int, C.c_int]
        L.edbref_qcalc_calQ.argtypes = [C.c_void_p, _dp, _dp]
        L.edbref_qcalc_copyB.argtypes = [C.c_void_p, _dp]
        L.edbref_qcalc_free.argtypes = [C.c_void_p]
        L.edbref_funF.restype = C.c_double
        L.edbref_funF.argtypes = [C.c_int, C.c_double, C.c_double]
        L.edbref_filtering.restype = C.c_double
        L.edbref_filtering.argtypes = [C.c_int, C.c_int]
        L.edbref_efix_new.restype = C.c_void_p
        L.edbref_efix_new.argtypes = [C.c_int, C.c_double]
        L.edbref_efix_free.argtypes = [C.c_void_p]
        L.edbref_efix_entropy.restype = C.c_double
        L.edbref_efix_entropy.argtypes = [C.c_void_p, C.c_int, _dp]
        L.edbref_efix_setaverage.argtypes = [C.c_void_p, C.c_int, _dp]
        L.edbref_efix_fixsol.argtypes = [C.c_void_p, C.c_int, _dp, C.c_double]
        L.edbref_efix_average.restype = C.c_double
        L.edbref_efix_average.argtypes = [C.c_void_p]
        L.edbref_fft.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp]
        L.edbref_ifft.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp]
        L.edbref_bkw_initial.argtypes = [C.c_int, C.c_double, C.c_double, _dp]
        L.edbref_bkw_entropy.restype = C.c_double
        L.edbref_bkw_entropy.argtypes = [C.c_int, C.c_double, _dp]
        L.edbref_bkw_run.restype = C.c_int
        L.edbref_bkw_run.argtypes = [C.c_int, C.c_double, C.c_int, C.c_double, C.c_double,
                                     C.c_double, C.c_double, C.c_int, _dp, _dp, C.c_char_p,
                                     C.c_int]
        L.edbref_time_calQ.restype = C.c_double
        L.edbref_time_calQ.argtypes = [C.c_void_p, _dp, _dp, C.c_int]

    def qcalc(self, N, alpha=0, filter=True):
        return RefQCalculator(self, N, alpha, filter)

    def funF(self, alpha, xi, eta):
        return self.L.edbref_funF(alpha, xi, eta)

    def filtering(self, N, beta):
        return self.L.edbref_filtering(N, beta)

    def fft(self, N, F):
        F = np.ascontiguousarray(F, dtype=np.complex128).reshape(-1).copy()
        out = np.empty_like(F)
        self.L.edbref_fft(N, N, N, _ptr(F.view(np.float64)), _ptr(out.view(np.float64)))
        return out

    def ifft(self, N, Fhat):
        Fhat = np.ascontiguousarray(Fhat, dtype=np.complex128).reshape(-1).copy()
        out = np.empty_like(Fhat)
        self.L.edbref_ifft(N, N, N, _ptr(out.view(np.float64)), _ptr(Fhat.view(np.float64)))
        return out

    def initial(self, N, R, t=0.0):
        F = np.empty(N ** 3, dtype=np.complex128)
        self.L.edbref_bkw_initial(N, R, t, _ptr(F.view(np.float64)))
        return F

    def calentropy(self, N, R, F):
        F = np.ascontiguousarray(F, dtype=np.complex128).reshape(-1)
        return self.L.edbref_bkw_entropy(N, R, _ptr(F.view(np.float64)))

    def fe_files(self, N, R, T0, TEnd, dt, fix, slice_name):
        """BKW3D::FEuler + outV1Direction of the compiled reference in the
        current directory: writes F.dat and slice_name there."""
        self.L.edbref_bkw_fe_files.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double,
                                               C.c_double, C.c_int, C.c_char_p]
        rc = self.L.edbref_bkw_fe_files(N, float(R), float(T0), float(TEnd), float(dt),
                                        int(bool(fix)), slice_name.encode())
        assert rc == 0

    def run(self, N, R, scheme, T0, TEnd, dt, beta=1.0, fix=True, log_cap=1 << 20):
        nq = N ** 3
        Fhat = np.empty(nq, dtype=np.complex128)
        F = np.empty(nq, dtype=np.complex128)
        buf = C.create_string_buffer(log_cap)
        sch = SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        rc = self.L.edbref_bkw_run(N, R, sch, T0, TEnd, dt, beta, int(bool(fix)),
                                   _ptr(Fhat.view(np.float64)), _ptr(F.view(np.float64)),
                                   buf, log_cap)
        assert rc == 0
        return Fhat, F, buf.value.decode()

    def run_from(self, N, R, scheme, F0, T0, TEnd, dt, checks):
        """RK4 or SSP3 step sequence of the reference's objects from the given
        real-space initial data (edbref_run_from).  Returns (Fhat, F) at the
        1-based steps in ``checks`` (arrays of shape [len(checks), N^3]) and the
        per-step entropy before / after the fix rule."""
        nq = N ** 3
        F0 = np.ascontiguousarray(F0, dtype=np.complex128).reshape(-1)
        chk = np.ascontiguousarray(checks, dtype=np.int32)
        Fh = np.empty((chk.size, nq), dtype=np.complex128)
        F = np.empty((chk.size, nq), dtype=np.complex128)
        cap = int(chk.max()) + 16
        raw = np.empty(cap)
        fixed = np.empty(cap)
        sch = SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        fn = self.L.edbref_run_from
        fn.restype = C.c_int
        fn.argtypes = [C.c_int, C.c_double, C.c_int, _dp, C.c_double, C.c_double, C.c_double,
                       C.c_int, _ip, _dp, _dp, _dp, _dp, C.c_int]
        n = fn(N, float(R), sch, _ptr(F0.view(np.float64)), float(T0), float(TEnd), float(dt),
               chk.size, chk.ctypes.data_as(_ip), _ptr(Fh.view(np.float64)),
               _ptr(F.view(np.float64)), _ptr(raw), _ptr(fixed), cap)
        assert n >= int(chk.max()), n
        return Fh, F, raw[:n].copy(), fixed[:n].copy()


class RefQCalculator:
    def __init__(self, ref: Reference, N, alpha, filter):
        self.ref = ref
        self.N = N
        self.h = ref.L.edbref_qcalc_new(N, alpha, int(bool(filter)))

    def calQ(self, fin):
        fin = np.ascontiguousarray(fin, dtype=np.complex128).reshape(-1)
        out = np.empty_like(fin)
        self.ref.L.edbref_qcalc_calQ(self.h, _ptr(fin.view(np.float64)),
                                     _ptr(out.view(np.float64)))
        return out

    def B(self):
        nq = self.N ** 3
        out = np.empty(nq * nq)
        self.ref.L.edbref_qcalc_copyB(self.h, _ptr(out))
        return out

    def time_calQ(self, fin, reps):
        fin = np.ascontiguousarray(fin, dtype=np.complex128).reshape(-1)
        out = np.empty_like(fin)
        return self.ref.L.edbref_time_calQ(self.h, _ptr(fin.view(np.float64)),
                                           _ptr(out.view(np.float64)), reps)

    def __del__(self):
        try:
            self.ref.L.edbref_qcalc_free(self.h)
        except Exception:
            pass


def parse_entropy_log(log: str):
    """Entropy columns printed by BKW3D integrators (BKW.h:431-444, 501-514).

    Returns a list of (t, entropy_raw, entropy_fixed_or_None) per step row.
    """
    rows = []
    for line in log.splitlines():
        if not line or line.startswith("#"):
            continue
        parts = line.split("\t")
        try:
            vals = [float(p) for p in parts if p.strip() not in ("", "-")]
        except ValueError:
            continue
        rows.append(vals)
    return rows
