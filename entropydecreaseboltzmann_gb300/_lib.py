"""ctypes binding of libedb.so (the C ABI declared in include/edb.h).

The library is built in-tree by ``entropydecreaseboltzmann_gb300.build.build()``.
There is no CPU fallback: importing this module when the library is missing
raises, and every compute call on a host without a usable GPU raises
``EdbError`` with status EDB_ECUDA.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libedb.so")

EDB_OK = 0
STATUS = {0: "EDB_OK", 1: "EDB_EINVAL", 2: "EDB_ENOMEM", 3: "EDB_ECUDA", 4: "EDB_ETIMEDOUT",
          5: "EDB_ENOTREADY", 6: "EDB_EBUSY", 7: "EDB_ENOTFOUND", 8: "EDB_ECANCELED",
          9: "EDB_ENONFINITE"}
INDEX_REFERENCE = 0
INDEX_ALIASED = 1
R_REFERENCE = 6.62132
SCHEME_FE, SCHEME_CFE, SCHEME_RK2, SCHEME_SSP3, SCHEME_RK4, SCHEME_DUFORT = range(6)
FP64_EMULATED, FP64_NATIVE, FP64_ONTHEFLY = 0, 1, 2


class EdbError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class QCalcDesc(C.Structure):
    _fields_ = [("N", C.c_int), ("gamma", C.c_double), ("L", C.c_double), ("filter", C.c_int),
                ("index_mode", C.c_int)]


class QCalcInfo(C.Structure):
    _fields_ = [("N", C.c_int), ("n", C.c_int), ("P", C.c_int), ("NQ", C.c_longlong),
                ("terms", C.c_longlong), ("B_bytes", C.c_longlong), ("has_B32", C.c_int)]


class SolverDesc(C.Structure):
    _fields_ = [("N", C.c_int), ("R", C.c_double), ("scheme", C.c_int), ("fix_entropy", C.c_int),
                ("beta", C.c_double), ("kernel", QCalcDesc), ("conserve", C.c_int),
                ("record_F", C.c_int)]


class BatchDesc(C.Structure):
    _fields_ = [("S", C.c_int), ("N", C.c_int), ("R", C.c_double), ("scheme", C.c_int),
                ("dt", C.c_double), ("fix_entropy", C.c_int), ("conserve", C.c_int)]


class ServerDesc(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("scheme", C.c_int), ("dt", C.c_double),
                ("fix_entropy", C.c_int), ("conserve", C.c_int), ("filter", C.c_int),
                ("max_live_per_group", C.c_int)]


class Request(C.Structure):
    _fields_ = [("N", C.c_int), ("gamma", C.c_double), ("R", C.c_double), ("steps", C.c_int),
                ("arrival_s", C.c_double), ("want_result", C.c_int)]


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_int), ("N", C.c_int), ("steps", C.c_int), ("t_arrival", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("live", C.c_longlong),
                ("queued", C.c_longlong), ("tts_p50_s", C.c_double), ("tts_p99_s", C.c_double),
                ("tts_mean_s", C.c_double), ("tts_max_s", C.c_double), ("wait_p50_s", C.c_double),
                ("wait_p99_s", C.c_double), ("first_arrival_s", C.c_double),
                ("last_done_s", C.c_double), ("throughput_rps", C.c_double),
                ("qhat_evals", C.c_double), ("qhat_evals_padded", C.c_double),
                ("qhat_evals_per_s", C.c_double), ("steps_launched", C.c_longlong),
                ("kernel_launches", C.c_longlong), ("hbm_bytes_peak", C.c_double),
                ("groups", C.c_int), ("refused", C.c_longlong), ("cancelled", C.c_longlong),
                ("failed", C.c_longlong)]


_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_vp = C.c_void_p
_ip = C.POINTER(C.c_int)


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with entropydecreaseboltzmann_gb300.build.build() "
            "(there is no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    sig = {
        "edb_last_error": (C.c_char_p, []),
        "edb_status_string": (C.c_char_p, [C.c_int]),
        "edb_version": (C.c_int, []),
        "edb_kernel_launch_count": (C.c_longlong, []),
        "edb_measure_fp32_peak": (C.c_int, [_dp]),
        "edb_measure_fp32x2_peak": (C.c_int, [_dp]),
        "edb_qcalc_desc_init": (C.c_int, [C.POINTER(QCalcDesc), C.c_int, C.c_int]),
        "edb_qcalc_create": (C.c_int, [C.POINTER(QCalcDesc), C.POINTER(_vp)]),
        "edb_qcalc_destroy": (C.c_int, [_vp]),
        "edb_qcalc_close_filter": (C.c_int, [_vp]),
        "edb_qcalc_genB": (C.c_int, [_vp]),
        "edb_qcalc_genB_compact": (C.c_int, [_vp]),
        "edb_qcalc_calQ": (C.c_int, [_vp, _dp, _dp]),
        "edb_qcalc_calQ_device": (C.c_int, [_vp, _vp, _vp, _vp]),
        "edb_qcalc_calQ_batch_f32_device": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
        "edb_qcalc_calQ_batch_f32_ex": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp,
                                                  _vp]),
        "edb_qcalc_autotune_batch": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _ip]),
        "edb_qcalc_calQ_batch_multi": (C.c_int, [C.c_int, _vp, _ip, _vp, _vp, C.c_int, _vp]),
        "edb_qcalc_autotune_batch_multi": (C.c_int, [C.c_int, _vp, _ip, _vp, _vp, _vp, _ip]),
        "edb_qcalc_batch_variants": (C.c_int, []),
        "edb_device_status": (C.c_int, [_ip, C.c_int]),
        "edb_set_wait_limit_ns": (C.c_int, [C.c_longlong]),
        "edb_qcalc_set_fp64_kernel": (C.c_int, [_vp, C.c_int]),
        "edb_qcalc_fp64_shape": (C.c_int, [_vp, C.c_int, _ip]),
        "edb_qcalc_fp64_shapes": (C.c_int, []),
        "edb_qcalc_copy_B": (C.c_int, [_vp, C.c_longlong, C.c_longlong, _dp]),
        "edb_qcalc_set_B": (C.c_int, [_vp, _dp]),
        "edb_qcalc_get_info": (C.c_int, [_vp, C.POINTER(QCalcInfo)]),
        "edb_fft3d_fft": (C.c_int, [C.c_int, C.c_int, C.c_int, _dp, _dp]),
        "edb_fft3d_ifft": (C.c_int, [C.c_int, C.c_int, C.c_int, _dp, _dp]),
        "edb_fft3d_device": (C.c_int, [C.c_int, C.c_int, _vp, _vp, C.c_int, C.c_int, _vp]),
        "edb_efix_create": (C.c_int, [C.c_int, C.c_double, C.POINTER(_vp)]),
        "edb_efix_destroy": (C.c_int, [_vp]),
        "edb_efix_set_average": (C.c_int, [_vp, C.c_int, _dp]),
        "edb_efix_entropy": (C.c_int, [_vp, C.c_int, _dp, _dp]),
        "edb_efix_fixsol": (C.c_int, [_vp, C.c_int, _dp, C.c_double]),
        "edb_efix_get_average": (C.c_int, [_vp, _dp, _ip]),
        "edb_solver_create": (C.c_int, [C.POINTER(SolverDesc), C.POINTER(_vp)]),
        "edb_solver_destroy": (C.c_int, [_vp]),
        "edb_solver_set_initial": (C.c_int, [_vp, _dp]),
        "edb_solver_run": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double, _ip]),
        "edb_solver_get": (C.c_int, [_vp, _dp, _dp]),
        "edb_solver_trace": (C.c_int, [_vp, _dp, _dp, C.c_int, _ip]),
        "edb_solver_F_history": (C.c_int, [_vp, _dp, C.c_int, _ip]),
        "edb_solver_write_F_dat": (C.c_int, [_vp, C.c_char_p]),
        "edb_solver_out_v1_direction": (C.c_int, [_vp, C.c_char_p]),
        "edb_batch_create": (C.c_int, [_vp, C.POINTER(BatchDesc), C.POINTER(_vp)]),
        "edb_batch_destroy": (C.c_int, [_vp]),
        "edb_batch_load": (C.c_int, [_vp, _dp]),
        "edb_batch_load_device": (C.c_int, [_vp, _vp, _vp]),
        "edb_batch_step": (C.c_int, [_vp, C.c_int, _vp]),
        "edb_batch_read": (C.c_int, [_vp, _dp, _dp]),
        "edb_batch_read_device": (C.c_int, [_vp, _vp, _vp]),
        "edb_batch_entropy": (C.c_int, [_vp, _dp, _dp]),
        "edb_batch_load_async": (C.c_int, [_vp, _dp]),
        "edb_batch_step_async": (C.c_int, [_vp, C.c_int]),
        "edb_batch_read_async": (C.c_int, [_vp, _dp]),
        "edb_batch_sync": (C.c_int, [_vp]),
        "edb_cells_transport_x_device": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double,
                                                   C.c_double, _vp, _vp, _vp]),
        "edb_batch_moments": (C.c_int, [_vp, _dp, _dp]),
        "edb_batch_launches_per_step": (C.c_int, [_vp, _ip]),
        "edb_qcalc_genB_f32": (C.c_int, [_vp]),
        "edb_funF": (C.c_int, [C.c_int, C.c_longlong, _dp, _dp, _dp]),
        "edb_filtering": (C.c_int, [C.c_int, C.c_longlong, _ip, _dp]),
        "edb_server_create": (C.c_int, [C.POINTER(ServerDesc), C.POINTER(_vp)]),
        "edb_server_destroy": (C.c_int, [_vp]),
        "edb_server_prepare": (C.c_int, [_vp, C.c_int, C.c_double, C.c_double]),
        "edb_server_submit": (C.c_int, [_vp, C.POINTER(Request), _dp, C.POINTER(C.c_longlong)]),
        "edb_server_run": (C.c_int, [_vp, C.c_double]),
        "edb_server_start": (C.c_int, [_vp]),
        "edb_server_stop": (C.c_int, [_vp]),
        "edb_server_wait": (C.c_int, [_vp, C.c_longlong, C.c_double]),
        "edb_server_cancel": (C.c_int, [_vp, C.c_longlong]),
        "edb_server_result": (C.c_int, [_vp, C.c_longlong, _dp, _dp, C.POINTER(RequestInfo)]),
        "edb_server_get_stats": (C.c_int, [_vp, C.POINTER(ServerStats)]),
        "edb_server_clock": (C.c_int, [_vp, _dp]),
        "edb_moments_hat_device": (C.c_int, [C.c_int, C.c_int, C.c_double, _vp, _vp, _vp]),
        "edb_moments_project_device": (C.c_int, [C.c_int, C.c_int, C.c_double, _vp, _vp, _vp]),
        "edb_maxwellian_fit_device": (C.c_int, [C.c_int, C.c_int, C.c_double, _vp, _vp, _vp,
                                                _vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


lib = _load()


def check(status: int) -> None:
    if status != EDB_OK:
        raise EdbError(status, lib.edb_last_error().decode(errors="replace"))


def dptr(a: np.ndarray):
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data_as(_dp)


def devptr(x) -> int:
    """Device address of a torch tensor, or an int address as is."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def stream_ptr(stream) -> int:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream
