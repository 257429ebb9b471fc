"""One launch over several (N, gamma) tables (edb_qcalc_calQ_batch_multi,
edb_qcalc_autotune_batch_multi).

Each CTA reads its table's descriptor by index; a table's CTAs run exactly as
its own launch would (same tile shape, pipeline depth and CTA order), so the
results must equal the per-table batched kernel bit for bit, and the FP32
tolerance against the FP64 oracle (relative L2 <= 5e-6) carries over.
"""
import numpy as np
import pytest

from oracle.oracle import INDEX_ALIASED

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def edb():
    import entropydecreaseboltzmann_gb300 as e

    return e


def rel_l2(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def _inputs(N, S, seed):
    import torch

    rng = np.random.default_rng(seed)
    f = rng.standard_normal((S, N ** 3)) + 1j * rng.standard_normal((S, N ** 3))
    return f, torch.from_numpy(f.astype(np.complex64)).cuda()


def test_grouped_equals_per_table(edb, oracle):
    import torch

    mix = [(8, 0.0, 5), (12, 1.0, 17), (16, 0.5, 1), (16, 0.0, 33), (24, 1.0, 9), (8, 0.5, 40),
           (20, 0.0, 3)]
    tabs, ref = [], []
    for i, (N, gamma, S) in enumerate(mix):
        q = edb.QCalculator(N, int(gamma), gamma=gamma, L=6.0, filter=False,
                            index_mode=INDEX_ALIASED)
        q.genB()
        fh, fin = _inputs(N, S, 70 + i)
        out = torch.full_like(fin, float("nan"))
        tabs.append((q, S, fin, out, fh, gamma))
        one = torch.empty_like(fin)
        q.calQ_batch_f32_ex(S, 4, 1, None, fin, one)
        ref.append(one)
    for v in range(5):  # every plain-layout variant, and the auto rule
        for t in tabs:
            t[3].fill_(float("nan"))
        edb.QCalculator.calQ_batch_multi([t[:4] for t in tabs], variant=v)
        torch.cuda.synchronize()
        for (q, S, fin, out, fh, _), one in zip(tabs, ref):
            assert torch.equal(out, one), (v, q.N, S)
    best = edb.QCalculator.autotune_batch_multi([t[:4] for t in tabs])
    assert 0 <= best <= 4
    for t in tabs:
        t[3].fill_(float("nan"))
    edb.QCalculator.calQ_batch_multi([t[:4] for t in tabs])
    torch.cuda.synchronize()
    for (q, S, fin, out, fh, _), one in zip(tabs, ref):
        assert torch.equal(out, one), (q.N, S)
    # the FP32 tolerance against the oracle on one solve of two tables
    for q, S, fin, out, fh, gamma in (tabs[1], tabs[2]):
        Bo = oracle.genB(q.N, gamma, 6.0, False, INDEX_ALIASED)
        Qo = oracle.calQ(q.N, Bo, fh[S - 1], INDEX_ALIASED)
        assert rel_l2(out[S - 1].cpu().numpy(), Qo) <= 5e-6
    assert edb.device_status() == 0


def test_grouped_sixteen_tables_one_handle(edb):
    """The descriptor array's full size: 16 entries (the same handle may
    appear more than once, each entry with its own buffers)."""
    import torch

    q = edb.QCalculator(12, 0, L=6.0, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    tabs, ref = [], []
    for i in range(16):
        S = 1 + 3 * i
        _, fin = _inputs(12, S, 90 + i)
        out = torch.empty_like(fin)
        one = torch.empty_like(fin)
        q.calQ_batch_f32_ex(S, 4, 1, None, fin, one)
        tabs.append((q, S, fin, out))
        ref.append(one)
    edb.QCalculator.calQ_batch_multi(tabs)
    torch.cuda.synchronize()
    for t, one in zip(tabs, ref):
        assert torch.equal(t[3], one)


def test_grouped_refusals(edb):
    import torch

    q8 = edb.QCalculator(8, 0, L=6.0, filter=False, index_mode=INDEX_ALIASED)
    q8.genB()
    _, fin = _inputs(8, 2, 1)
    out = torch.empty_like(fin)
    with pytest.raises(edb.EdbError) as e:  # more than 16 tables
        edb.QCalculator.calQ_batch_multi([(q8, 2, fin, out)] * 17)
    assert e.value.status == 1
    with pytest.raises(edb.EdbError) as e:  # no tables
        edb.QCalculator.calQ_batch_multi([])
    assert e.value.status == 1
    q9 = edb.QCalculator(9, 0, L=6.0, filter=False, index_mode=INDEX_ALIASED)
    q9.genB()
    _, fin9 = _inputs(9, 2, 2)
    with pytest.raises(edb.EdbError) as e:  # N % 4 != 0: no tensor-copy path
        edb.QCalculator.calQ_batch_multi([(q8, 2, fin, out), (q9, 2, fin9, torch.empty_like(fin9))])
    assert e.value.status == 1
    qn = edb.QCalculator(8, 0, L=6.0, filter=False, index_mode=INDEX_ALIASED)
    with pytest.raises(edb.EdbError) as e:  # no table yet
        edb.QCalculator.calQ_batch_multi([(qn, 2, fin, out)])
    assert e.value.status == 5
    with pytest.raises(edb.EdbError) as e:
        edb.QCalculator.calQ_batch_multi([(q8, 0, fin, out)])
    assert e.value.status == 1
    for v in (5, 9, 10):  # pair-layout variants and unknown ones
        with pytest.raises(edb.EdbError) as e:
            edb.QCalculator.calQ_batch_multi([(q8, 2, fin, out)], variant=v)
        assert e.value.status == 1
