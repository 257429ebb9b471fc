"""Bounded device waits: a wait that runs out is drained, reported and leaves
the context usable.

Every mbarrier wait inside the two Q-hat kernels has a limit (200 ms by
default).  edb_set_wait_limit_ns(0) makes every wait run out at once, so the
first wait of every warp runs out while the copies issued before it are in
flight.  The kernel then stops issuing copies, waits (with its own drain limit) for
the copies it did issue, sets its status word and returns without writing its
output.  Nothing here faults or hangs the GPU: the failure is a timeout the
kernel handles itself.
"""
import numpy as np
import pytest

from oracle.oracle import INDEX_ALIASED

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def edb():
    import entropydecreaseboltzmann_gb300 as e

    return e


def test_wait_timeout_is_drained_reported_and_recovers(edb):
    import torch

    from entropydecreaseboltzmann_gb300 import data

    N, L, S = 24, 7.0, 64  # N % 4 == 0: both kernels stage through TMA copies
    F0, _, _ = data.bkw_bump_batch(S, N, L, seed=11)
    fh = np.fft.fftn(F0.reshape(S, N, N, N), axes=(1, 2, 3)).reshape(S, -1)
    q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    fin = torch.from_numpy(fh.astype(np.complex64)).cuda()
    good = torch.empty_like(fin)
    q.calQ_batch_f32(S, fin, good)
    torch.cuda.synchronize()
    good64 = q.calQ(None, fh[0])
    assert edb.device_status(clear=True) == 0

    edb.set_wait_limit_ns(0)
    try:
        out = torch.zeros_like(fin)
        q.calQ_batch_f32(S, fin, out)  # stream-ordered: the caller reads the status
        torch.cuda.synchronize()
        st = edb.device_status(clear=True)
        assert st & 1, st
        with pytest.raises(edb.EdbError) as e:  # synchronous: EDB_ETIMEDOUT itself
            q.calQ(None, fh[0])
        assert e.value.status == 4
    finally:
        edb.set_wait_limit_ns(-1)
    # the synchronous call read and cleared the words
    assert edb.device_status(clear=True) == 0

    again = torch.empty_like(fin)
    q.calQ_batch_f32(S, fin, again)
    torch.cuda.synchronize()
    assert torch.equal(again, good)
    assert np.array_equal(q.calQ(None, fh[0]), good64)
    assert edb.device_status(clear=True) == 0


def test_wait_timeout_in_the_persistent_grouped_launch(edb):
    """The grouped launch's persistent CTAs stop pulling work items once a
    wait of theirs runs out; the status word is set and the next launch gives
    the earlier bits."""
    import torch

    qs, tabs = [], []
    for N, S in ((16, 40), (8, 33)):
        q = edb.QCalculator(N, 0, L=6.0, filter=False, index_mode=INDEX_ALIASED)
        q.genB()
        rng = np.random.default_rng(N)
        f = rng.standard_normal((S, N ** 3)) + 1j * rng.standard_normal((S, N ** 3))
        fin = torch.from_numpy(f.astype(np.complex64)).cuda()
        qs.append(q)
        tabs.append((q, S, fin, torch.empty_like(fin)))
    edb.QCalculator.calQ_batch_multi(tabs, variant=4)
    torch.cuda.synchronize()
    good = [t[3].clone() for t in tabs]
    assert edb.device_status(clear=True) == 0
    edb.set_wait_limit_ns(0)
    try:
        edb.QCalculator.calQ_batch_multi(tabs, variant=4)
        torch.cuda.synchronize()
        st = edb.device_status(clear=True)
        assert st & 1, st
    finally:
        edb.set_wait_limit_ns(-1)
    edb.QCalculator.calQ_batch_multi(tabs, variant=4)
    torch.cuda.synchronize()
    for t, g in zip(tabs, good):
        assert torch.equal(t[3], g)
    assert edb.device_status(clear=True) == 0
