"""Host-side logic of the serving workloads (no GPU): the seeded request
streams have the stated distributions, and initial data have mass 1."""
import math

import numpy as np

from entropydecreaseboltzmann_gb300 import data, serving


def test_stream_requests_distribution():
    reqs = serving.stream_requests(rate=2000.0, duration=1.0, seed=5)
    n = len(reqs)
    assert abs(n - 2000) < 5 * math.sqrt(2000)            # Poisson count
    t = np.array([r["arrival"] for r in reqs])
    assert np.all(np.diff(t) > 0) and t[-1] < 1.0
    gaps = np.diff(t)
    assert abs(gaps.mean() - 1 / 2000) < 0.1 / 2000       # exponential gaps
    Ns = np.array([r["N"] for r in reqs])
    for N, p in ((16, 0.5), (24, 0.3), (32, 0.2)):
        assert abs(np.mean(Ns == N) - p) < 0.04
    assert {r["L"] for r in reqs if r["N"] == 24} == {7.0}
    steps = np.array([r["steps"] for r in reqs])
    assert steps.min() >= 20 and steps.max() <= 500
    # log-uniform: the median is near sqrt(20 * 500) = 100
    assert 80 <= np.median(steps) <= 125
    bkw = [r for r in reqs if r["bkw_t0"] is not None]
    assert abs(len(bkw) / n - 0.05) < 0.015
    assert all(r["gamma"] == 0.0 and 5.5 <= r["bkw_t0"] <= 8.0 for r in bkw)
    assert {r["gamma"] for r in reqs} <= {0.0, 1.0}


def test_stream_requests_are_seeded():
    a = serving.stream_requests(100.0, 1.0, seed=9)
    b = serving.stream_requests(100.0, 1.0, seed=9)
    assert a == b


def test_uneven_requests():
    reqs = serving.uneven_requests(512, seed=1)
    assert len(reqs) == 1536
    for N in (16, 24, 32):
        sub = [r for r in reqs if r["N"] == N]
        assert len(sub) == 512 and {r["L"] for r in sub} == {serving.L_OF_N[N]}
    assert {r["gamma"] for r in reqs} == {0.0, 0.5, 1.0}
    steps = [r["steps"] for r in reqs]
    assert min(steps) >= 20 and max(steps) <= 200
    assert all(r["arrival"] == 0.0 for r in reqs)


def test_initial_data_mass_one():
    for r in serving.stream_requests(200.0, 0.2, seed=3)[:12]:
        f = serving.initial_data(r)
        assert f.shape == (r["N"] ** 3,)
        assert abs(data.mass(f, r["N"], r["L"]) - 1.0) < 1e-6
