"""The real-space output after a step with the fix rule on.

The reference's post-step rule (BKW.h:497-515 for RK4) computes F = ifft(Fhat),
its entropy, and on an entropy rise rewrites F with EntropyFix::FixSol; Fhat
is left alone.  F is the output (the files, the next rule's entropy).  So the
batch's read, moments and the served result return that F, and it differs
from ifft(Fhat) where the fix acted.

Data: a two-Maxwellian mixture on N = 12, L = 8.9755 whose entropy rises by
3.8e-4 on the second RK4 step (found by a seeded search with the oracle; the
spectral grid's small values cross FixSol's 1e-6 cut-off), so the fix acts on
the last step of a 2-step run.

Tolerances: entropies recomputed in numpy from the returned arrays against the
batch's own trace, relative 1e-12 (summation order only); the fixed F against
the oracle's FP64 run of the reference rule, relative L2 <= 1e-6 (FP32 Q-hat).
"""
import numpy as np
import pytest

from oracle.oracle import INDEX_ALIASED

pytestmark = pytest.mark.gpu

N, L, DT = 12, 8.97548252617662, 0.01
COMPS = [((1.7957746997510613, -0.1598194427636157, 1.0309153812331657), 1.1456185823289522,
          0.6234497281574163),
         ((1.14314280285523, -0.34137660257731683, 0.9379342871549174), 1.5089428925825747,
          0.9456477492907027)]


@pytest.fixture(scope="module")
def edb():
    import entropydecreaseboltzmann_gb300 as e

    return e


def _f0():
    v = -L + 2 * L * np.arange(N) / N
    X, Y, Z = np.meshgrid(v, v, v, indexing="ij")
    f = sum(w * np.exp(-((X - u[0]) ** 2 + (Y - u[1]) ** 2 + (Z - u[2]) ** 2) / (2 * T))
            / (2 * np.pi * T) ** 1.5 for u, T, w in COMPS)
    return f.reshape(-1)


def _entropy(f):
    """calEntropy (BKW.h:140-161): sum of f log f - f over |f| >= 1e-6, times (2L)^3 / N^3."""
    f = np.asarray(f, dtype=np.float64)
    big = np.abs(f) >= 1.0e-6
    val = np.zeros_like(f)
    val[big] = f[big] * np.log(f[big]) - f[big]
    return val.sum() * (2 * L) ** 3 / N ** 3


def _batch(edb, q, steps, f0):
    b = edb.BatchSolver(q, 2, L, edb.SCHEME_RK4, DT, fix_entropy=True)
    b.load(np.stack([f0, f0]))
    b.step(steps)
    return b


def test_read_returns_the_fixed_output(edb, oracle):
    f0 = _f0()
    q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    b = _batch(edb, q, 2, f0)
    raw, fixed = b.entropy()
    assert raw[0] != fixed[0]  # the fix acted on the last step
    F, Fh = b.read(real=True, fhat=True)
    F_state = np.fft.ifftn(Fh[0].reshape(N, N, N)).real.reshape(-1)
    assert np.max(np.abs(F[0] - F_state)) > 0.0
    assert abs(_entropy(F[0]) - fixed[0]) <= 1e-12 * abs(fixed[0])
    assert abs(_entropy(F_state) - raw[0]) <= 1e-12 * abs(raw[0])
    # the read does not move the state: a second read gives the same bits
    assert np.array_equal(b.read(real=True), F)
    # the reference rule in FP64 (the oracle) gives the same fixed output
    _, Fo, ro, fo = oracle.run(N, L, "RK4", 0.0, 1.5 * DT, DT, fix=True, F0=f0,
                               mode=INDEX_ALIASED, Rb=L, filter=False)
    assert ro[-1] != fo[-1]
    assert np.linalg.norm(F[0] - Fo.real) <= 1e-6 * np.linalg.norm(Fo.real)
    # moments come from the same output
    m, H = b.moments()
    assert abs(H[0] - fixed[0]) <= 1e-12 * abs(fixed[0])
    # device read equals host read
    import torch

    d = torch.empty(2 * N ** 3, dtype=torch.float64, device="cuda")
    b.read_device(d)
    assert np.array_equal(d.cpu().numpy().reshape(2, -1), F)


def test_read_after_load_and_without_fix(edb):
    """Before any step f is the loaded data; with the fix off f = ifft(Fhat)."""
    f0 = _f0()
    q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    b = edb.BatchSolver(q, 2, L, edb.SCHEME_RK4, DT, fix_entropy=False)
    b.load(np.stack([f0, f0]))
    assert np.array_equal(b.read(real=True)[0], f0)
    raw, fixed = b.entropy()
    assert np.isnan(raw).all() and np.isnan(fixed).all()
    b.step(2)
    F, Fh = b.read(real=True, fhat=True)
    F_state = np.fft.ifftn(Fh[0].reshape(N, N, N)).real.reshape(-1)
    assert np.max(np.abs(F[0] - F_state)) <= 1e-15 * np.max(np.abs(F_state)) * N ** 3


def test_served_result_is_the_fixed_output(edb):
    """The server returns the same fixed output as the batch (same kernel,
    scheme and table; its l1-plane chunking changes the last bits of Q-hat, so
    the fix's bisection on beta may land one step of its 1e-10 resolution
    apart: relative L2 <= 1e-9)."""
    f0 = _f0()
    q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    b = _batch(edb, q, 2, f0)
    F_b = b.read(real=True)[0]
    raw, fixed = b.entropy()
    srv = edb.Server(hbm_budget_bytes=4e9, scheme=edb.SCHEME_RK4, dt=DT, fix_entropy=True)
    rid = srv.submit(N, 0.0, L, 2, f0, want_result=True)
    srv.run()
    F, _ = srv.result(rid)
    assert np.linalg.norm(F - F_b) <= 1e-9 * np.linalg.norm(F_b)
    # the served F carries the fixed entropy, not the raw one
    H = _entropy(F)
    assert abs(H - fixed[0]) < 0.1 * abs(raw[0] - fixed[0])
    srv.close()
