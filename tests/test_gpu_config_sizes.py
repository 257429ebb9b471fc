"""GPU parity at the workloads' sizes against the compiled reference.

Fixtures: tests/golden/reference_golden_configs.npz (tests/golden/make_golden.py,
from the reference's own QCalculator / fft3d / EntropyFix / BKW3D objects).

Tolerances
  FP64 trajectories (Fhat, and F where no fix acts): relative L2 <= 1e-11
    after up to 100 RK4 steps.  The kernels sum in another order than the
    reference's loops (about 1e-15 per evaluation); the stage updates round
    where the reference's do.
  F after EntropyFix: relative L2 <= 1e-9.  FixSol bisects on beta to 1e-10;
    a last-bit difference in an entropy can move one bisection decision,
    which moves beta (and F) by up to that resolution.
  Entropy traces: relative 1e-11 before the fix, 1e-9 after it.  NaN
    entries (log of negative F under the even-N loops) must sit at the same
    steps.
  FP64 calQ at N = 24 / 25: relative L2 <= 1e-12 (both FP64 kernels).
  BKW L-inf (ALIASED mode, N = 16, L = 6, filter off): <= 3e-5 at every one of
    the 100 steps.  That is the grid's discretisation floor (the oracle's own
    FP64 run reaches 2.59e-5 at t = 1); the trajectory equals the oracle's
    to 1e-11 after 10 steps.
"""
import os

import numpy as np
import pytest

from oracle.oracle import INDEX_ALIASED, R_REFERENCE

pytestmark = pytest.mark.gpu

CFG = os.path.join(os.path.dirname(__file__), "golden", "reference_golden_configs.npz")


@pytest.fixture(scope="module")
def edb():
    import entropydecreaseboltzmann_gb300 as e

    return e


@pytest.fixture(scope="module")
def cfg():
    return np.load(CFG)


def rel_l2(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def _run(edb, N, R, scheme, F0, nsteps, dt, **kernel):
    """One run of the device-resident integrator for exactly nsteps steps
    (`do { t += dt } while (t < TEnd)` with TEnd = (nsteps - 1/2) dt)."""
    b = edb.BKW3D(N, R, **kernel)
    b.setFixEntropy(True)
    b.setInitial(F0)
    getattr(b, scheme)(0.0, (nsteps - 0.5) * dt, dt)
    assert b.nsteps == nsteps
    return b


@pytest.mark.parametrize("tag", ["bkw", "sin"])
def test_config1_rk4_reference_mode_matches_reference(edb, cfg, tag):
    """The testBKW3D case on RK4 in the reference's index mode: N = 16 on
    [-6, 6]^3, QCalculator(N0, 0) (Maxwell, filter on, R = 6.62132 in rval),
    dt = 0.01, from the BKW profile at t0 = 5.5 (100 steps) or the reference's
    own sinusoid (10 steps).  Fhat at every checkpoint, F and both entropy
    traces at the last one."""
    F0 = cfg[f"cfg1_{tag}_F0"]
    checks = [int(c) for c in cfg[f"cfg1_{tag}_checks"]]
    for i, n in enumerate(checks):
        b = _run(edb, 16, 6.0, "RK4", F0, n, 0.01)
        assert rel_l2(b.Fhat, cfg[f"cfg1_{tag}_Fhat"][i]) <= 1e-11, n
    raw, fixed = cfg[f"cfg1_{tag}_ent_raw"], cfg[f"cfg1_{tag}_ent_fixed"]
    np.testing.assert_allclose(b.entropy_raw, raw, rtol=1e-11, equal_nan=True)
    np.testing.assert_allclose(b.entropy_fixed, fixed, rtol=1e-9, equal_nan=True)
    tol = 1e-11 if np.array_equal(raw, fixed, equal_nan=True) else 1e-9
    assert rel_l2(b.F, cfg[f"cfg1_{tag}_F"]) <= tol


def test_config1_rk4_aliased_bkw_linf_every_step(edb, oracle):
    """The same case in the aliased index mode with the box's own L in the
    kernel scale and the filter off: L-inf of Re F against the exact BKW
    solution after every step, and the trajectory against the oracle."""
    from entropydecreaseboltzmann_gb300 import data

    N, L, dt, steps = 16, 6.0, 0.01, 100
    f0 = data.bkw_grid(N, L, 5.5)
    kern = dict(L=L, filter=False, index_mode=INDEX_ALIASED)
    b = edb.BKW3D(N, L, record_F=True, **kern)
    b.setInitial(f0)
    b.RK4(0.0, (steps - 0.5) * dt, dt)
    assert b.nsteps == steps
    linf = [float(np.max(np.abs(b.F_history[s] - data.bkw_grid(N, L, 5.5 + (s + 1) * dt))))
            for s in range(steps)]
    print("BKW L-inf by step (N=16, FP64):", " ".join(f"{e:.2e}" for e in linf))
    assert max(linf) <= 3e-5, max(linf)
    assert linf[0] <= 1e-6
    b10 = _run(edb, N, L, "RK4", f0, 10, dt, **kern)
    Fo, _, _, _ = oracle.run(N, L, "RK4", 0.0, 9.5 * dt, dt, fix=True, F0=f0, mode=INDEX_ALIASED,
                             Rb=L, filter=False)
    assert rel_l2(b10.Fhat, Fo) <= 1e-11


@pytest.mark.parametrize("N", [15, 16, 17])
def test_ssp3_fix_matches_reference(edb, cfg, N):
    """SSP3 with the fix rule (BKW.h:387-449), 10 steps of dt = 0.005 on the
    reference's [-6.62132, 6.62132]^3: N = 16 from the sinusoid (the fix acts
    on steps 2-10), N = 15 and 17 from a two-Maxwellian mixture."""
    b = _run(edb, N, R_REFERENCE, "SSP3", cfg[f"ssp3_N{N}_F0"], 10, 0.005)
    assert rel_l2(b.Fhat, cfg[f"ssp3_N{N}_Fhat"]) <= 1e-11
    raw, fixed = cfg[f"ssp3_N{N}_ent_raw"], cfg[f"ssp3_N{N}_ent_fixed"]
    np.testing.assert_allclose(b.entropy_raw, raw, rtol=1e-11, equal_nan=True)
    np.testing.assert_allclose(b.entropy_fixed, fixed, rtol=1e-9, equal_nan=True)
    fix_acted = not np.array_equal(raw, fixed, equal_nan=True)
    assert rel_l2(b.F, cfg[f"ssp3_N{N}_F"]) <= (1e-9 if fix_acted else 1e-11)
    if N == 16:
        assert fix_acted


@pytest.mark.parametrize("N,alpha,filt", [(24, 0, 1), (25, 1, 0)])
def test_calQ_fp64_at_workload_N_matches_reference(edb, cfg, N, alpha, filt):
    """QCalculator::calQ of the reference at N = 24 (its loops, even N) and
    N = 25 (odd: the aliased sum), both FP64 kernels."""
    tag = f"N{N}_a{alpha}_f{filt}"
    q = edb.QCalculator(N, alpha, filter=bool(filt))
    q.genB()
    fin = cfg[f"calq_in_{tag}"]
    want = cfg[f"calq_out_{tag}"]
    for kind in (0, 1):
        q.set_fp64_kernel(kind)
        assert rel_l2(q.calQ(None, fin), want) <= 1e-12, kind
