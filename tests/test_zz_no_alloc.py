"""The allocation-free FP64 collision sum, called through the C ABI.

edb_calQ_fp64_noalloc exists for callers that may not call cudaMalloc (a host
that owns a fixed device pool, a plugin inside it, a real-time loop).  Here
the caller's memory is torch tensors; the function must give the same Q-hat
as the handle-based entry point edb_qcalc_calQ_device, within the FP64 parity
tolerance, on two calls in a row (the second reuses the fixed scratch array
the first left behind), and the second call must not change the device's free
memory.  This file sorts last so a run that stops at its first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative L2, the FP64 parity tolerance of the other GPU tests


def _noalloc_fn():
    from entropydecreaseboltzmann_gb300 import _lib

    fn = _lib.lib.edb_calQ_fp64_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return fn, _lib


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("N,mode", [(9, 0), (16, 0), (17, 1)])
def test_noalloc_calQ_matches_handle_path_twice(N, mode):
    import torch

    import entropydecreaseboltzmann_gb300 as edb

    fn, _lib = _noalloc_fn()
    q = edb.QCalculator(N, 0, index_mode=mode)
    q.genB()
    d_B = torch.from_numpy(q.B()).cuda()  # the table, in memory the caller owns
    rng = np.random.default_rng(100 + N)
    stream = torch.cuda.current_stream()
    for call in range(2):
        fin = rng.standard_normal(N ** 3) + 1j * rng.standard_normal(N ** 3)
        d_fin = torch.from_numpy(fin).cuda()
        d_ref = torch.empty_like(d_fin)
        d_out = torch.full_like(d_fin, complex(np.nan, np.nan))
        q.calQ_device(d_fin, d_ref, stream)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        st = fn(N, mode, d_B.data_ptr(), d_fin.data_ptr(), d_out.data_ptr(), stream.cuda_stream)
        assert st == 0, _lib.lib.edb_last_error().decode()
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        if call == 1:
            assert free1 == free0, "the second call changed the device's free memory"
        got, ref = d_out.cpu().numpy(), d_ref.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert _rel_l2(got, ref) <= TOL, (call, _rel_l2(got, ref))


def test_noalloc_rejects_out_of_range_sizes():
    import torch

    fn, _lib = _noalloc_fn()
    x = torch.zeros(2, dtype=torch.complex128, device="cuda")
    for N in (2, 65, 100):
        st = fn(N, 0, x.data_ptr(), x.data_ptr(), x.data_ptr(), None)
        assert st == 1  # EDB_EINVAL
        assert b"N must be in [3, 64]" in _lib.lib.edb_last_error()
    assert fn(9, 0, None, x.data_ptr(), x.data_ptr(), None) == 1
