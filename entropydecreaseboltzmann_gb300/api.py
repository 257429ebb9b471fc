"""Python mirror of the reference's classes over the C ABI of libedb.so.

Names, argument meaning and call order follow the reference:
QCalculator (CalQ/QCalculator.h:17-62), fft3d (CalQ/fft3d.h:17-49),
EntropyFix (CalQ/EntropyFix.h:13-46) and BKW3D (CalQ/BKW.h:22-62).
Host arrays are numpy (complex128 for c_type, float64 for r_type), N^3
entries in FFTW order.  Device buffers are torch tensors or raw addresses.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (INDEX_REFERENCE, R_REFERENCE, SCHEME_CFE, SCHEME_DUFORT, SCHEME_FE,
                   SCHEME_RK2, SCHEME_RK4, SCHEME_SSP3, BatchDesc, QCalcDesc, QCalcInfo,
                   Request, RequestInfo, ServerDesc, ServerStats, SolverDesc, check, devptr, dptr,
                   lib, stream_ptr)


def device_status(clear: bool = True) -> int:
    """Nonzero when a bounded wait inside a Q-hat kernel ran out (bit 0: the
    batched kernel, bit 1: the double-float FP64 kernel)."""
    v = C.c_int()
    check(lib.edb_device_status(C.byref(v), int(clear)))
    return v.value


def set_wait_limit_ns(ns: int) -> None:
    """Limit of each bounded wait inside the Q-hat kernels in nanoseconds
    (ns < 0: the 200 ms default; 0: every wait runs out at once).  For tests
    of the timeout path."""
    check(lib.edb_set_wait_limit_ns(int(ns)))


def kernel_launch_count() -> int:
    """Kernels libedb.so has launched in this process (graph replays included)."""
    return int(lib.edb_kernel_launch_count())


def _c128(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.complex128).reshape(-1)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} complex entries, got {a.size}")
    return a


class QCalculator:
    """QCalculator<std::complex<double>, double>(N, alpha) on the GPU.

    ``L`` (box half-width in rval), ``gamma`` (real VHS exponent) and
    ``index_mode`` generalise constants the reference hard-codes; the
    defaults reproduce it (QCalculator.h:31-34, 176).
    """

    def __init__(self, N: int, alpha: int = 0, *, gamma: float | None = None,
                 L: float = R_REFERENCE, filter: bool = True,
                 index_mode: int = INDEX_REFERENCE):
        d = QCalcDesc()
        check(lib.edb_qcalc_desc_init(C.byref(d), int(N), int(alpha)))
        if gamma is not None:
            d.gamma = float(gamma)
        d.L = float(L)
        d.filter = int(bool(filter))
        d.index_mode = int(index_mode)
        self.desc = d
        self.N = int(N)
        self.NQ = self.N ** 3
        h = C.c_void_p()
        check(lib.edb_qcalc_create(C.byref(d), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def closeFilter(self):
        check(lib.edb_qcalc_close_filter(self._h))
        self.desc.filter = 0

    def genB(self):
        check(lib.edb_qcalc_genB(self._h))

    def genB_compact(self):
        """genB without the N^6 table: only the small tables the on-the-fly
        FP64 kernel reads (aliased index shifts: ALIASED mode or odd N)."""
        check(lib.edb_qcalc_genB_compact(self._h))

    def funF(self, xi, eta):
        """funF(xi, eta) (QCalculator.h:76-106) for this calculator's alpha,
        evaluated on the device; scalars or arrays."""
        x = np.ascontiguousarray(np.atleast_1d(xi), dtype=np.float64)
        e = np.ascontiguousarray(np.broadcast_to(np.atleast_1d(eta), x.shape), dtype=np.float64)
        out = np.empty_like(x)
        check(lib.edb_funF(int(round(self.desc.gamma)) if float(self.desc.gamma).is_integer()
                           else -1, x.size, dptr(x), dptr(e), dptr(out)))
        return float(out[0]) if np.ndim(xi) == 0 else out

    def filtering(self, beta):
        """filtering(beta) (QCalculator.h:67-74), evaluated on the device."""
        b = np.ascontiguousarray(np.atleast_1d(beta), dtype=np.int32)
        out = np.empty(b.shape, dtype=np.float64)
        check(lib.edb_filtering(self.N, b.size, b.ctypes.data_as(C.POINTER(C.c_int)), dptr(out)))
        return float(out[0]) if np.ndim(beta) == 0 else out

    def calQ(self, Qout, fin):
        """calQ(Qout, fin) (QCalculator.h:231-257): Qout <- Q-hat(fin), FP64."""
        fin = _c128(fin, self.NQ)
        if Qout is None:
            Qout = np.empty(self.NQ, dtype=np.complex128)
        if Qout.dtype != np.complex128 or not Qout.flags["C_CONTIGUOUS"] or Qout.size != self.NQ:
            raise ValueError("Qout must be a contiguous complex128 array of N^3 entries")
        check(lib.edb_qcalc_calQ(self._h, dptr(fin.view(np.float64)),
                                 dptr(Qout.reshape(-1).view(np.float64))))
        return Qout

    def calQ_device(self, d_fin, d_Q, stream=None):
        check(lib.edb_qcalc_calQ_device(self._h, devptr(d_fin), devptr(d_Q), stream_ptr(stream)))

    def calQ_batch_f32(self, S, d_fin, d_Q, stream=None):
        check(lib.edb_qcalc_calQ_batch_f32_device(self._h, int(S), devptr(d_fin), devptr(d_Q),
                                                  stream_ptr(stream)))

    def calQ_batch_f32_ex(self, S, variant, chunks, d_partial, d_fin, d_Q, stream=None):
        """Batched kernel with an explicit variant (0 .. batch_variants() - 1;
        0, 1: 16-solve groups; 2: 4-solve groups; 3, 4: 4 outputs per thread;
        5-9: the same on a solve-pair copy of the input) and l1-plane chunk
        count (d_partial: chunks x S x N^3 x 16 bytes on the device when
        chunks > 1)."""
        check(lib.edb_qcalc_calQ_batch_f32_ex(self._h, int(S), int(variant), int(chunks),
                                              devptr(d_partial), devptr(d_fin), devptr(d_Q),
                                              stream_ptr(stream)))

    @staticmethod
    def _multi_args(tables):
        n = len(tables)
        return (n, (C.c_void_p * n)(*[t[0]._h for t in tables]),
                (C.c_int * n)(*[int(t[1]) for t in tables]),
                (C.c_void_p * n)(*[devptr(t[2]) for t in tables]),
                (C.c_void_p * n)(*[devptr(t[3]) for t in tables]))

    @staticmethod
    def calQ_batch_multi(tables, variant=-1, stream=None):
        """Batched Q-hat of several tables in one launch: tables is a list of
        (QCalculator, S, d_fin, d_Q), 1 to 16 entries, each handle in ALIASED
        mode after genB with N % 4 == 0.  variant: 0-4, or -1 for the heaviest
        table's autotuned one.  Same bits as calQ_batch_f32_ex with one chunk,
        table by table."""
        check(lib.edb_qcalc_calQ_batch_multi(*QCalculator._multi_args(tables), int(variant),
                                             stream_ptr(stream)))

    @staticmethod
    def autotune_batch_multi(tables, stream=None):
        """The fastest plain-layout variant for this grouped launch."""
        v = C.c_int()
        check(lib.edb_qcalc_autotune_batch_multi(*QCalculator._multi_args(tables),
                                                 stream_ptr(stream), C.byref(v)))
        return v.value

    def set_fp64_kernel(self, kind):
        """0 = FP64-accurate double-float on the FP32 pipe (default), 1 = native FP64,
        2 = double-float with the pair entries formed on the fly (no N^6 table)."""
        check(lib.edb_qcalc_set_fp64_kernel(self._h, int(kind)))

    def fp64_shape(self, shape=-1):
        """Launch shape of the double-float FP64 kernel (timed at genB); shape
        >= 0 overrides it.  Returns the shape in use."""
        v = C.c_int()
        check(lib.edb_qcalc_fp64_shape(self._h, int(shape), C.byref(v)))
        return v.value

    def autotune_batch(self, S, d_fin, d_Q, stream=None):
        """Pick the fastest batched-kernel variant for S solves; returns its index."""
        v = C.c_int()
        check(lib.edb_qcalc_autotune_batch(self._h, int(S), devptr(d_fin), devptr(d_Q),
                                           stream_ptr(stream), C.byref(v)))
        return v.value

    def B(self, first=0, count=None):
        total = self.NQ * self.NQ
        count = total - first if count is None else count
        out = np.empty(count, dtype=np.float64)
        check(lib.edb_qcalc_copy_B(self._h, int(first), int(count), dptr(out)))
        return out

    def set_B(self, B):
        B = np.ascontiguousarray(B, dtype=np.float64).reshape(-1)
        if B.size != self.NQ * self.NQ:
            raise ValueError("B must hold N^6 entries")
        check(lib.edb_qcalc_set_B(self._h, dptr(B)))

    def info(self):
        i = QCalcInfo()
        check(lib.edb_qcalc_get_info(self._h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in QCalcInfo._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib.edb_qcalc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class fft3d:
    """fft3d (CalQ/fft3d.h:17-49) on the GPU, FP64, host buffers."""

    def fft(self, Nx, Ny, Nz, re, fre):
        """fre <- unnormalised forward DFT of re (fft3d.h:25-30)."""
        n = Nx * Ny * Nz
        re = _c128(re, n)
        if fre.dtype != np.complex128 or fre.size != n or not fre.flags["C_CONTIGUOUS"]:
            raise ValueError("fre must be a contiguous complex128 array")
        check(lib.edb_fft3d_fft(Nx, Ny, Nz, dptr(re.view(np.float64)),
                                dptr(fre.reshape(-1).view(np.float64))))
        return fre

    def ifft(self, Nx, Ny, Nz, re, fre):
        """re <- backward DFT of fre times 1/(Nx Ny Nz) (fft3d.h:32-48)."""
        n = Nx * Ny * Nz
        fre = _c128(fre, n)
        if re.dtype != np.complex128 or re.size != n or not re.flags["C_CONTIGUOUS"]:
            raise ValueError("re must be a contiguous complex128 array")
        check(lib.edb_fft3d_ifft(Nx, Ny, Nz, dptr(re.reshape(-1).view(np.float64)),
                                 dptr(fre.view(np.float64))))
        return re

    DOUBLE_FLOAT = 2  # EDB_DFT_DOUBLE_FLOAT

    @staticmethod
    def device(N, batch, d_in, d_out, inverse=False, fp32=False, stream=None):
        """fp32: False / 0 complex128 data in FP64, True / 1 complex64 data,
        fft3d.DOUBLE_FLOAT complex128 data with double-float passes."""
        check(lib.edb_fft3d_device(int(N), int(batch), devptr(d_in), devptr(d_out),
                                   int(bool(inverse)), int(fp32), stream_ptr(stream)))


class EntropyFix:
    """EntropyFix<int, double>(Nt, eps) (CalQ/EntropyFix.h) on the GPU."""

    def __init__(self, Nt: int, eps: float = 1.0e-10):
        h = C.c_void_p()
        check(lib.edb_efix_create(int(Nt), float(eps), C.byref(h)))
        self._h = h
        self.Nt = int(Nt)
        self.eps = float(eps)

    @staticmethod
    def _args(args):
        # (fin) or (Nf, fin) like the reference's vector / pointer overloads
        if len(args) == 1:
            f = args[0]
            return len(f), f
        return int(args[0]), args[1]

    def setAverage(self, *args):
        Nf, f = self._args(args)
        f = np.ascontiguousarray(f, dtype=np.float64)
        check(lib.edb_efix_set_average(self._h, Nf, dptr(f)))

    def EntropyCal(self, *args):
        Nf, f = self._args(args)
        f = np.ascontiguousarray(f, dtype=np.float64)
        H = C.c_double()
        check(lib.edb_efix_entropy(self._h, Nf, dptr(f), C.byref(H)))
        return H.value

    def FixSol(self, *args):
        """FixSol(fin, aim) or FixSol(Nf, fin, aim): fin is modified in place."""
        if len(args) == 2:
            f, aim = args
            Nf = len(f)
        else:
            Nf, f, aim = args
        if not (isinstance(f, np.ndarray) and f.dtype == np.float64 and f.flags["C_CONTIGUOUS"]):
            raise ValueError("fin must be a contiguous float64 numpy array (modified in place)")
        check(lib.edb_efix_fixsol(self._h, int(Nf), dptr(f), float(aim)))
        return f

    @property
    def average(self):
        a = C.c_double()
        fl = C.c_int()
        check(lib.edb_efix_get_average(self._h, C.byref(a), C.byref(fl)))
        return a.value

    def __del__(self):
        try:
            if self._h:
                lib.edb_efix_destroy(self._h)
                self._h = None
        except Exception:
            pass


class BKW3D:
    """BKW3D<c_type, r_type>(N0, R) (CalQ/BKW.h:22-62) with every integrator
    loop (calQ stages, stage updates, ifft, entropy, fix) on the device.

    The kernel table defaults to the reference's QCalculator(N0, 0): Maxwell
    molecules, R = 6.62132 in rval, filter on, REFERENCE index mode.
    """

    def __init__(self, N0: int, R: float, *, gamma: float = 0.0, L: float = R_REFERENCE,
                 filter: bool = True, index_mode: int = INDEX_REFERENCE, conserve: bool = False,
                 record_F: bool = False):
        self.N0 = int(N0)
        # keep Re F after every step (F_history, write_F_dat)
        self.record_F = bool(record_F)
        self.F_history = None
        self._h = None
        # conservative mode (no reference counterpart): moments projected back
        # after every step, moment-preserving entropy fix fed back into Fhat
        self.conserve = bool(conserve)
        self.R = float(R)
        self.N3d = self.N0 ** 3
        self.kernel = dict(gamma=float(gamma), L=float(L), filter=bool(filter),
                           index_mode=int(index_mode))
        self.FixEntropy = False
        self._F0 = None
        self.F = None
        self.Fhat = None
        self.entropy_raw = None
        self.entropy_fixed = None
        self.nsteps = 0

    def setFixEntropy(self, fix: bool = True):
        self.FixEntropy = bool(fix)

    def setInitial(self, F0):
        """Real-space initial data (N^3 complex or real); None = setInitialValue's sinusoid."""
        self._F0 = None if F0 is None else _c128(F0, self.N3d)

    def _run(self, scheme, T0, TEnd, dt, beta=1.0):
        d = SolverDesc()
        d.N = self.N0
        d.R = self.R
        d.scheme = scheme
        d.fix_entropy = int(self.FixEntropy)
        d.beta = float(beta)
        d.kernel.N = self.N0
        d.kernel.gamma = self.kernel["gamma"]
        d.kernel.L = self.kernel["L"]
        d.kernel.filter = int(self.kernel["filter"])
        d.kernel.index_mode = self.kernel["index_mode"]
        d.conserve = int(self.conserve)
        d.record_F = int(self.record_F)
        self._release()
        h = C.c_void_p()
        check(lib.edb_solver_create(C.byref(d), C.byref(h)))
        ok = False
        try:
            F0p = None if self._F0 is None else dptr(self._F0.view(np.float64))
            check(lib.edb_solver_set_initial(h, F0p))
            ns = C.c_int()
            check(lib.edb_solver_run(h, float(T0), float(TEnd), float(dt), C.byref(ns)))
            self.nsteps = ns.value
            self.Fhat = np.empty(self.N3d, dtype=np.complex128)
            self.F = np.empty(self.N3d, dtype=np.complex128)
            check(lib.edb_solver_get(h, dptr(self.Fhat.view(np.float64)),
                                     dptr(self.F.view(np.float64))))
            raw = np.empty(ns.value)
            fixed = np.empty(ns.value)
            n = C.c_int()
            check(lib.edb_solver_trace(h, dptr(raw), dptr(fixed), ns.value, C.byref(n)))
            self.entropy_raw, self.entropy_fixed = raw, fixed
            if self.record_F:
                hist = np.empty((ns.value, self.N3d))
                check(lib.edb_solver_F_history(h, dptr(hist), ns.value, C.byref(n)))
                self.F_history = hist
            ok = True
        finally:
            if ok:
                self._h = h  # kept for the output writers
            else:
                lib.edb_solver_destroy(h)
        return self

    def write_F_dat(self, filename: str = "F.dat"):
        """The per-step F.dat rows of BKW3D::FEuler (BKW.h:217-249), written in the
        reference's stream format (needs record_F=True)."""
        if self._h is None:
            raise RuntimeError("run an integrator first")
        check(lib.edb_solver_write_F_dat(self._h, str(filename).encode()))

    def outV1Direction(self, filename: str):
        """BKW3D::outV1Direction (BKW.h:163-180): x, Re F and funExact along v1
        through the grid centre, in the reference's format."""
        if self._h is None:
            raise RuntimeError("run an integrator first")
        check(lib.edb_solver_out_v1_direction(self._h, str(filename).encode()))

    @staticmethod
    def slice_filename(N: int, dt: float) -> str:
        """testBKW3D.cpp:44: "N" + std::to_string(N) + ".dt" + std::to_string(dt) + ".dat"."""
        return f"N{int(N)}.dt{float(dt):f}.dat"

    def _release(self):
        if getattr(self, "_h", None):
            lib.edb_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass

    def FEuler(self, T0, TEnd, dt):
        return self._run(SCHEME_FE, T0, TEnd, dt)

    def CFE(self, T0, TEnd, dt, beta):
        return self._run(SCHEME_CFE, T0, TEnd, dt, beta)

    def RK2(self, T0, TEnd, dt):
        return self._run(SCHEME_RK2, T0, TEnd, dt)

    def SSP3(self, T0, TEnd, dt):
        return self._run(SCHEME_SSP3, T0, TEnd, dt)

    def RK4(self, T0, TEnd, dt):
        return self._run(SCHEME_RK4, T0, TEnd, dt)

    def DUFORT(self, T0, TEnd, dt, beta):
        return self._run(SCHEME_DUFORT, T0, TEnd, dt, beta)


class BatchSolver:
    """S independent solves sharing one ALIASED kernel table.

    Q-hat runs in complex FP32 with compensated sums (edb_qcalc_calQ_batch_f32_device);
    the RK state, stage updates, inverse transforms, moments and the entropy
    rule run in FP64.  One CUDA graph launch advances every solve by one step.
    """

    def __init__(self, qcalc: QCalculator, S: int, R: float, scheme: int = SCHEME_RK4,
                 dt: float = 0.01, fix_entropy: bool = False, conserve: bool = False):
        d = BatchDesc()
        d.conserve = int(bool(conserve))
        d.S = int(S)
        d.N = qcalc.N
        d.R = float(R)
        d.scheme = int(scheme)
        d.dt = float(dt)
        d.fix_entropy = int(bool(fix_entropy))
        h = C.c_void_p()
        check(lib.edb_batch_create(qcalc.handle, C.byref(d), C.byref(h)))
        self._h = h
        self.q = qcalc
        self.S = int(S)
        self.N = qcalc.N
        self.NQ = self.N ** 3
        self._pending = []  # host buffers of queued asynchronous copies

    def load(self, F0_real):
        F0 = np.ascontiguousarray(F0_real, dtype=np.float64).reshape(-1)
        if F0.size != self.S * self.NQ:
            raise ValueError("expected S x N^3 real values")
        check(lib.edb_batch_load(self._h, dptr(F0)))

    def load_device(self, d_F0_real, stream=None):
        check(lib.edb_batch_load_device(self._h, devptr(d_F0_real), stream_ptr(stream)))

    def step(self, nsteps=1, stream=None):
        check(lib.edb_batch_step(self._h, int(nsteps), stream_ptr(stream)))

    def read(self, real=True, fhat=False, out=None):
        """Real-space f (S x N^3) and/or Fhat.  out: a C-contiguous float64 array of
        S x N^3 to receive f directly (e.g. pinned host memory), instead of a new one.
        With fix_entropy on, f after a step is the step's output after the fix
        rule (the reference's F), which differs from ifft(Fhat) where the fix
        acted."""
        if real and out is not None:
            if out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or out.size != self.S * self.NQ:
                raise ValueError("out must be a contiguous float64 array of S x N^3")
            F = out.reshape(-1)
        else:
            F = np.empty(self.S * self.NQ) if real else None
        Fh = np.empty(self.S * self.NQ, dtype=np.complex128) if fhat else None
        check(lib.edb_batch_read(self._h, None if F is None else dptr(F),
                                 None if Fh is None else dptr(Fh.view(np.float64))))
        out = []
        if real:
            out.append(F.reshape(self.S, self.NQ))
        if fhat:
            out.append(Fh.reshape(self.S, self.NQ))
        return out[0] if len(out) == 1 else tuple(out)

    def load_async(self, F0_real):
        """Queued load from a C-contiguous float64 host array (pinned for the
        copies to overlap); keep it alive and unchanged until sync()."""
        if F0_real.dtype != np.float64 or not F0_real.flags["C_CONTIGUOUS"] \
                or F0_real.size != self.S * self.NQ:
            raise ValueError("expected a contiguous float64 array of S x N^3")
        self._pending.append(F0_real)
        check(lib.edb_batch_load_async(self._h, dptr(F0_real.reshape(-1))))

    def step_async(self, nsteps=1):
        check(lib.edb_batch_step_async(self._h, int(nsteps)))

    def read_async(self, out):
        """Queued read of real-space f into a C-contiguous float64 host array
        of S x N^3 (pinned for the copies to overlap); valid after sync()."""
        if out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] \
                or out.size != self.S * self.NQ:
            raise ValueError("out must be a contiguous float64 array of S x N^3")
        self._pending.append(out)
        check(lib.edb_batch_read_async(self._h, dptr(out.reshape(-1))))

    def sync(self):
        check(lib.edb_batch_sync(self._h))
        self._pending.clear()

    def read_device(self, d_F_real, stream=None):
        """Real-space f (S x N^3 float64) into a device buffer (torch tensor or address)."""
        check(lib.edb_batch_read_device(self._h, devptr(d_F_real), stream_ptr(stream)))

    def entropy(self):
        """(raw, fixed): each solve's entropy after its last step, before and
        after the fix rule (NaN before the first step)."""
        raw = np.empty(self.S)
        fixed = np.empty(self.S)
        check(lib.edb_batch_entropy(self._h, dptr(raw), dptr(fixed)))
        return raw, fixed

    def moments(self):
        m = np.empty(self.S * 5)
        H = np.empty(self.S)
        check(lib.edb_batch_moments(self._h, dptr(m), dptr(H)))
        return m.reshape(self.S, 5), H

    def launches_per_step(self):
        n = C.c_int()
        check(lib.edb_batch_launches_per_step(self._h, C.byref(n)))
        return n.value

    def __del__(self):
        try:
            if self._h:
                lib.edb_batch_destroy(self._h)
                self._h = None
        except Exception:
            pass


class CellSolver:
    """Spatially inhomogeneous use: df/dt + v1 df/dx = Q(f) on a periodic 1-D
    grid of C cells [0, Lx), each cell holding a velocity distribution on
    [-R, R]^3 (N^3 points), all sharing one ALIASED kernel table (no reference
    counterpart: the reference solves the homogeneous equation only).

    The state is a C x N^3 float64 device tensor, cells-major.  ``collide``
    advances every cell's homogeneous collision step (a BatchSolver with one
    solve per cell: FP32 compensated Q-hat, FP64 state), ``transport`` streams
    freely in x (edb_cells_transport_x_device), and ``strang_step`` does
    transport dt/2, collide dt, transport dt/2."""

    def __init__(self, qcalc: QCalculator, C: int, R: float, Lx: float, scheme: int = SCHEME_RK4,
                 dt: float = 0.01, fix_entropy: bool = False, conserve: bool = False):
        self.C, self.N, self.R, self.Lx, self.dt = int(C), qcalc.N, float(R), float(Lx), float(dt)
        self.batch = BatchSolver(qcalc, C, R, scheme, dt, fix_entropy=fix_entropy,
                                 conserve=conserve)

    def transport(self, d_f, d_out, dt, stream=None):
        """d_out <- free streaming of d_f over dt (both C x N^3, distinct)."""
        check(lib.edb_cells_transport_x_device(self.C, self.N, self.R, self.Lx, float(dt),
                                               devptr(d_f), devptr(d_out), stream_ptr(stream)))

    def collide(self, d_f, nsteps=1, stream=None):
        """In place: every cell's distribution advanced nsteps collision steps."""
        self.batch.load_device(d_f, stream)
        self.batch.step(int(nsteps), stream)
        self.batch.read_device(d_f, stream)

    def strang_step(self, d_f, d_tmp, stream=None):
        """One Strang step of length dt, in place on d_f (d_tmp: scratch of the same shape)."""
        self.transport(d_f, d_tmp, 0.5 * self.dt, stream)
        self.collide(d_tmp, 1, stream)
        self.transport(d_tmp, d_f, 0.5 * self.dt, stream)


# ---------------------------------------------------------- serving engine

class Server:
    """Device-resident request loop with continuous batching (no reference
    counterpart).  Requests are independent solves grouped by kernel table
    (N, gamma, R); all use the server's scheme and dt.  See include/edb.h."""

    def __init__(self, hbm_budget_bytes: float = 80e9, scheme: int = SCHEME_RK4, dt: float = 0.01,
                 fix_entropy: bool = False, conserve: bool = False, filter: bool = False,
                 max_live_per_group: int = 0):
        d = ServerDesc()
        d.hbm_budget_bytes = float(hbm_budget_bytes)
        d.scheme = int(scheme)
        d.dt = float(dt)
        d.fix_entropy = int(bool(fix_entropy))
        d.conserve = int(bool(conserve))
        d.filter = int(bool(filter))
        d.max_live_per_group = int(max_live_per_group)
        h = C.c_void_p()
        check(lib.edb_server_create(C.byref(d), C.byref(h)))
        self._h = h
        self._N = {}

    def prepare(self, N: int, gamma: float, R: float):
        check(lib.edb_server_prepare(self._h, int(N), float(gamma), float(R)))

    def submit(self, N: int, gamma: float, R: float, steps: int, F0_real, arrival_s: float = -1.0,
               want_result: bool = False) -> int:
        F0 = np.ascontiguousarray(F0_real, dtype=np.float64).reshape(-1)
        if F0.size != N ** 3:
            raise ValueError("expected N^3 real values")
        r = Request()
        r.N, r.gamma, r.R, r.steps = int(N), float(gamma), float(R), int(steps)
        r.arrival_s = float(arrival_s)
        r.want_result = int(bool(want_result))
        rid = C.c_longlong()
        check(lib.edb_server_submit(self._h, C.byref(r), dptr(F0), C.byref(rid)))
        self._N[rid.value] = int(N)
        return rid.value

    def run(self, max_wall_s: float = 0.0):
        """Run the loop on this thread until every submitted request is done."""
        check(lib.edb_server_run(self._h, float(max_wall_s)))

    def start(self):
        """Run the loop on a background thread; submit() may then be called at any time."""
        check(lib.edb_server_start(self._h))

    def stop(self):
        check(lib.edb_server_stop(self._h))

    def wait(self, rid: int, timeout_s: float = 0.0):
        """Block until request rid is done (timeout_s <= 0: no limit)."""
        check(lib.edb_server_wait(self._h, int(rid), float(timeout_s)))

    def cancel(self, rid: int):
        """Cancel request rid: dropped if queued, retired (slot freed) at the end
        of its step in flight if running; wait() then raises EDB_ECANCELED."""
        check(lib.edb_server_cancel(self._h, int(rid)))

    def info(self, rid: int) -> dict:
        i = RequestInfo()
        check(lib.edb_server_result(self._h, int(rid), None, None, C.byref(i)))
        # state: 0 queued, 1 running, 2 done, 3 refused, 4 cancelled, 5 failed
        return {"state": i.state, "N": i.N, "steps": i.steps, "t_arrival": i.t_arrival,
                "t_admit": i.t_admit, "t_done": i.t_done}

    def result(self, rid: int):
        """(f real N^3, Fhat complex N^3) of a finished request kept with want_result."""
        NQ = self._N[int(rid)] ** 3
        F = np.empty(NQ)
        Fh = np.empty(NQ, dtype=np.complex128)
        check(lib.edb_server_result(self._h, int(rid), dptr(F), dptr(Fh.view(np.float64)), None))
        return F, Fh

    def clock(self) -> float:
        """Server clock in seconds (0 before the first run)."""
        t = C.c_double()
        check(lib.edb_server_clock(self._h, C.byref(t)))
        return t.value

    def stats(self) -> dict:
        st = ServerStats()
        check(lib.edb_server_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib.edb_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------ conservation
# No reference counterpart: the moment functionals of conservative mode.  The
# arrays are torch CUDA tensors (complex128, S x N^3, FFTW order) or device
# addresses.

def moments_hat(N: int, R: float, Fhat, out, S: int = 1, stream=None):
    """Grid moments h^3 sum Re F {1, v1, v2, v3, |v|^2} of S solves from Fhat
    into `out` (S x 5 float64 on the device)."""
    check(lib.edb_moments_hat_device(int(N), int(S), float(R), devptr(Fhat), devptr(out),
                                     stream_ptr(stream)))


def moments_project(N: int, R: float, Fhat, m0, S: int = 1, stream=None):
    """Minimum-norm correction of Fhat (in place) onto the moments m0 (S x 5)."""
    check(lib.edb_moments_project_device(int(N), int(S), float(R), devptr(Fhat), devptr(m0),
                                         stream_ptr(stream)))


def maxwellian_fit(N: int, R: float, F, theta, status, S: int = 1, stream=None):
    """Discrete Maxwellian of Re F per solve, written into Im F; theta (S x 5
    float64) = (a, b1, b2, b3, c) of exp(a + b.v + c|v|^2); status (S int32) =
    Newton iterations or -1."""
    check(lib.edb_maxwellian_fit_device(int(N), int(S), float(R), devptr(F), devptr(theta),
                                        devptr(status), stream_ptr(stream)))
