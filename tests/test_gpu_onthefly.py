"""FP64 collision sum with the kernel table formed on the fly (EDB_FP64_ONTHEFLY,
edb_qcalc_genB_compact): no N^6 table is built or read.

Tolerances
  Against the oracle (the reference's loops) and against the streamed
  double-float kernel: relative L2 <= 1e-12 (every kernel rounds in its own
  order; the pair entry is formed in double-float arithmetic, about 2^-48
  relative, instead of being rounded once in FP64).
  Where the oracle's full table would be too large (N = 32, 48), against the
  oracle's direct evaluation of the aliased sum at sampled modes: <= 1e-12 up
  to N = 32.  At N = 48, beyond what the reference's own loops can run (their
  int table index overflows from N = 36), <= 1e-11: the double-float running
  sums lose about 2^-48 per term, and the error grows with the N^3 / 2 pair
  terms per output (measured 3.7e-12 here; the streamed double-float kernel
  is at 1.2e-12 against native FP64 already at N = 40).  Native FP64
  (kernel 1) stays at 1e-15 there.
"""
import numpy as np
import pytest

from oracle.oracle import INDEX_ALIASED, INDEX_REFERENCE, R_REFERENCE

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def edb():
    import entropydecreaseboltzmann_gb300 as e

    return e


def rel_l2(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


@pytest.mark.parametrize("N,mode,gamma,filt", [
    (5, INDEX_ALIASED, 0.0, True), (6, INDEX_ALIASED, 1.0, False), (8, INDEX_ALIASED, 0.5, False),
    (9, INDEX_ALIASED, 1.0, True), (7, INDEX_REFERENCE, 0.0, True), (9, INDEX_REFERENCE, 1.0, False),
    (12, INDEX_ALIASED, 0.0, False), (16, INDEX_ALIASED, 1.0, True), (17, INDEX_REFERENCE, 0.0, True)])
def test_onthefly_matches_oracle_and_streamed(edb, oracle, N, mode, gamma, filt):
    rng = np.random.default_rng(500 + N)
    fin = rng.standard_normal(N ** 3) + 1j * rng.standard_normal(N ** 3)
    L = 6.0 if mode == INDEX_ALIASED else R_REFERENCE
    q = edb.QCalculator(N, int(gamma), gamma=gamma, L=L, filter=filt, index_mode=mode)
    q.genB()
    Qo = oracle.calQ(N, oracle.genB(N, gamma, L, filt, mode), fin, mode)
    q.set_fp64_kernel(0)
    Qs = q.calQ(None, fin)
    q.set_fp64_kernel(2)
    Qf = q.calQ(None, fin)
    assert rel_l2(Qf, Qo) <= 1e-12
    assert rel_l2(Qf, Qs) <= 1e-12
    # the compact tables alone give the same bits
    qc = edb.QCalculator(N, int(gamma), gamma=gamma, L=L, filter=filt, index_mode=mode)
    qc.genB_compact()
    assert np.array_equal(qc.calQ(None, fin), Qf)
    with pytest.raises(edb.EdbError) as e:  # no full table to copy
        qc.B(0, 4)
    assert e.value.status == 5


def test_onthefly_refuses_even_N_reference_mode(edb):
    q = edb.QCalculator(8, 0)  # REFERENCE mode, even N: no pair structure
    with pytest.raises(edb.EdbError) as e:
        q.genB_compact()
    assert e.value.status == 1


@pytest.mark.parametrize("N,L,gamma,tol", [(24, 7.0, 0.0, 1e-12), (32, 8.0, 1.0, 1e-12),
                                           (48, 8.0, 1.0, 1e-11)])
def test_onthefly_at_workload_N(edb, oracle, N, L, gamma, tol):
    """Compact tables only (the full FP64 table would be 1.5 GB, 8.6 GB and
    98 GB): against the oracle's direct aliased sum at 64 sampled modes, on a
    two-Maxwellian mixture; at N = 24 also against the streamed kernel."""
    from entropydecreaseboltzmann_gb300 import data

    f = data.two_maxwellians(N, L, seed=N)
    fin = np.fft.fftn(f.reshape(N, N, N)).reshape(-1)
    q = edb.QCalculator(N, int(gamma), gamma=gamma, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB_compact()
    Qf = q.calQ(None, fin)
    modes = np.random.default_rng(N).choice(N ** 3, 64, replace=False)
    Qd = oracle.direct_modes(N, fin, modes, gamma=gamma, R=L, filter=False)
    assert rel_l2(Qf[modes], Qd) <= tol
    if N == 24:
        qs = edb.QCalculator(N, int(gamma), gamma=gamma, L=L, filter=False,
                             index_mode=INDEX_ALIASED)
        qs.genB()
        assert rel_l2(Qf, qs.calQ(None, fin)) <= 1e-12
