"""GB300-native spectral collision step of the 3D space-homogeneous Boltzmann equation.

A from-scratch sm_103a implementation of the collision step of
YK2015/EntropyDecreaseBoltzmann behind the reference's own call surface:

* ``QCalculator(N, alpha)`` — genB / closeFilter / calQ (CalQ/QCalculator.h)
* ``fft3d``                 — fft / ifft (CalQ/fft3d.h)
* ``EntropyFix(Nt, eps)``   — EntropyCal / setAverage / FixSol (CalQ/EntropyFix.h)
* ``BKW3D(N, R)``           — FEuler / CFE / RK2 / SSP3 / RK4 / DUFORT (CalQ/BKW.h),
  run entirely on the device
* ``BatchSolver``           — many independent solves sharing one kernel table,
  Q-hat in complex FP32 with compensated sums, state and moments in FP64
* ``Server``                — device-resident request loop with continuous
  batching of independent solves grouped by kernel table

All compute runs in libedb.so (hand-written CUDA for sm_103a, C ABI in
include/edb.h).  There is no CPU fallback.
"""
from ._lib import (INDEX_ALIASED, INDEX_REFERENCE, R_REFERENCE, SCHEME_CFE, SCHEME_DUFORT,
                   SCHEME_FE, SCHEME_RK2, SCHEME_RK4, SCHEME_SSP3, EdbError, lib)
from .api import (BKW3D, BatchSolver, CellSolver, EntropyFix, QCalculator, Server,
                  device_status, fft3d,
                  kernel_launch_count, maxwellian_fit, moments_hat, moments_project,
                  set_wait_limit_ns)

__all__ = [
    "QCalculator", "fft3d", "EntropyFix", "BKW3D", "BatchSolver", "CellSolver", "EdbError",
    "INDEX_REFERENCE", "INDEX_ALIASED", "R_REFERENCE", "SCHEME_FE", "SCHEME_CFE", "SCHEME_RK2",
    "SCHEME_SSP3", "SCHEME_RK4", "SCHEME_DUFORT", "kernel_launch_count", "device_status", "lib",
    "moments_hat", "moments_project", "maxwellian_fit", "Server", "set_wait_limit_ns",
]
