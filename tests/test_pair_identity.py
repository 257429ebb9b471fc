"""The symmetric-pair form of the aliased Q-hat sum, checked on the CPU oracle.

Both Q-hat kernels of the ALIASED mode (the batched FP32 kernel and the
double-float FP64 kernel) read a pair table and visit half the l1 planes:
  Q_k = sum over l1 in [0, k1/2] u [k1+1, (k1+N)/2] (FFTW order) of
        P[l][k] f_l f_(k-l),   P[l][k] = B[l][k] + B[k-l][k]  (l1 != m1),
                               P[l][k] = B[l][k]              (l1 == m1).
This restates that in numpy on the oracle's own table and compares it with
the oracle's calQ (the reference's aliased loop): relative L2 <= 1e-13.
"""
import numpy as np
import pytest

from oracle.oracle import INDEX_ALIASED


@pytest.fixture(scope="module")
def oracle():
    from oracle.oracle import Oracle, build_oracle

    build_oracle()
    return Oracle()


def to_fftw(B, N):
    """Centred [l][k] table -> FFTW-order [lf][kf]."""
    n = (N - 1) // 2
    c = np.arange(N)
    f = (c - n) % N  # FFTW index of centred index c
    idx = (f[:, None, None] * N * N + f[None, :, None] * N + f[None, None, :]).reshape(-1)
    NQ = N ** 3
    out = np.empty((NQ, NQ))
    out[np.ix_(idx, idx)] = B.reshape(NQ, NQ)
    return out


def visited_planes(k1, N):
    return list(range(k1 // 2 + 1)) + list(range(k1 + 1, (k1 + N) // 2 + 1))


@pytest.mark.parametrize("N", [4, 5, 6, 7])
def test_pair_table_sum_equals_full_sum(oracle, N):
    rng = np.random.default_rng(100 + N)
    NQ = N ** 3
    B = oracle.genB(N, 1.0, 6.0, False, INDEX_ALIASED)
    fin = rng.standard_normal(NQ) + 1j * rng.standard_normal(NQ)
    want = oracle.calQ(N, B, fin, INDEX_ALIASED)
    Bf = to_fftw(B, N)
    v = np.array(np.unravel_index(np.arange(NQ), (N, N, N))).T  # FFTW index vectors
    got = np.zeros(NQ, dtype=complex)
    for k in range(NQ):
        m = (v[k] - v) % N  # partner of every l
        mflat = (m[:, 0] * N + m[:, 1]) * N + m[:, 2]
        l1, m1 = v[:, 0], m[:, 0]
        P = Bf[:, k] + np.where(l1 != m1, Bf[mflat, k], 0.0)
        keep = np.isin(l1, visited_planes(v[k][0], N))
        got[k] = np.sum(P[keep] * fin[keep] * fin[mflat[keep]])
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-13
    # every unordered pair {l, k - l} is visited once: count per k is half the
    # off-diagonal lines plus the diagonal planes' lines
    for k1 in range(N):
        vis = visited_planes(k1, N)
        diag = [a for a in range(N) if (2 * a - k1) % N == 0]
        assert sorted(vis) == sorted(set(vis))
        assert len(vis) == (N - len(diag)) // 2 + len(diag)
        assert all(a in vis for a in diag)
