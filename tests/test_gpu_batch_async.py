"""Asynchronous batch calls (edb_batch_load_async / step_async / read_async /
sync): the same bits as the synchronous calls, alone and with two batches
interleaved so that one's host copies overlap the other's steps."""
import numpy as np
import pytest

from oracle.oracle import INDEX_ALIASED

pytestmark = pytest.mark.gpu

N, L, S, DT = 12, 6.0, 5, 0.005


@pytest.fixture(scope="module")
def edb():
    import entropydecreaseboltzmann_gb300 as e

    return e


def _pinned(shape):
    import torch

    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


def _data(seed):
    from entropydecreaseboltzmann_gb300 import data

    f = _pinned((S, N ** 3))
    f[:] = data.maxwellian_mixture_batch(S, N, L, seed=seed)
    return f


def _sync_run(edb, q, f0, steps):
    b = edb.BatchSolver(q, S, L, edb.SCHEME_SSP3, DT, fix_entropy=True)
    b.load(f0)
    b.step(steps)
    return b.read(real=True).copy()


def test_async_equals_sync(edb):
    q = edb.QCalculator(N, 1, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    f0 = _data(7)
    want = _sync_run(edb, q, f0, 3)
    b = edb.BatchSolver(q, S, L, edb.SCHEME_SSP3, DT, fix_entropy=True)
    out = _pinned((S, N ** 3))
    b.load_async(f0)
    b.step_async(3)
    b.read_async(out)
    b.sync()
    assert np.array_equal(out, want)
    # again on the same batch (the load resets the state; the copies reuse
    # the staging buffer the step writes)
    out2 = _pinned((S, N ** 3))
    b.load_async(f0)
    b.step_async(3)
    b.read_async(out2)
    b.sync()
    assert np.array_equal(out2, want)


def test_two_batches_interleaved(edb):
    q = edb.QCalculator(N, 1, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    inputs = [_data(20 + i) for i in range(4)]
    want = [_sync_run(edb, q, f, 2) for f in inputs]
    bs = [edb.BatchSolver(q, S, L, edb.SCHEME_SSP3, DT, fix_entropy=True) for _ in range(2)]
    outs = [_pinned((S, N ** 3)) for _ in range(4)]
    for i, f in enumerate(inputs):
        b = bs[i % 2]  # a batch's next load queues behind its previous read
        b.load_async(f)
        b.step_async(2)
        b.read_async(outs[i])
    for b in bs:
        b.sync()
    for o, w in zip(outs, want):
        assert np.array_equal(o, w)
    assert edb.device_status() == 0
