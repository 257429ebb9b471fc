"""Serving engine on the GPU: continuous batching of independent solves.

Stated tolerance for "the same alone and in the mix": relative L2 of f and
Fhat <= 1e-12 (each solve's arithmetic depends only on its own slot; the
test also reports whether the results are bit-identical).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def edb():
    import entropydecreaseboltzmann_gb300 as e

    return e


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_result_same_alone_and_in_mix(edb):
    from entropydecreaseboltzmann_gb300 import data

    N, R, steps = 16, 6.0, 30
    f_probe = data.maxwellian_mixture_batch(1, N, R, seed=11)[0]
    # alone
    srv = edb.Server(hbm_budget_bytes=8e9, scheme=edb.SCHEME_RK4, dt=0.01)
    rid = srv.submit(N, 0.0, R, steps, f_probe, want_result=True)
    srv.run()
    F_alone, Fh_alone = srv.result(rid)
    srv.close()
    # in a mix: other N, gamma and horizons, arrivals spread over the run so
    # requests join while others are on the GPU
    rng = np.random.default_rng(5)
    srv = edb.Server(hbm_budget_bytes=8e9, scheme=edb.SCHEME_RK4, dt=0.01)
    srv.prepare(N, 0.0, R)
    srv.prepare(12, 1.0, 6.0)
    ids = []
    for j in range(40):
        n = int(rng.choice([12, 16]))
        g = float(rng.choice([0.0, 1.0]))
        f = data.maxwellian_mixture_batch(1, n, 6.0, seed=100 + j)[0]
        ids.append(srv.submit(n, g, 6.0, int(rng.integers(5, 60)), f,
                              arrival_s=float(rng.uniform(0, 0.05))))
    rid = srv.submit(N, 0.0, R, steps, f_probe, arrival_s=0.02, want_result=True)
    srv.run()
    F_mix, Fh_mix = srv.result(rid)
    st = srv.stats()
    assert st["completed"] == 41
    assert rel_l2(F_mix, F_alone) <= 1e-12
    assert rel_l2(Fh_mix, Fh_alone) <= 1e-12
    print("bit-identical:", bool(np.array_equal(F_mix, F_alone)))
    srv.close()


def test_server_matches_batch_solver(edb):
    """A served request equals the same solve in a BatchSolver (same scheme,
    table and FP32-compensated kernel)."""
    from entropydecreaseboltzmann_gb300 import data
    from oracle.oracle import INDEX_ALIASED

    N, R, steps = 12, 6.0, 20
    f0 = data.maxwellian_mixture_batch(3, N, R, seed=21)
    q = edb.QCalculator(N, 1, L=R, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    b = edb.BatchSolver(q, 3, R, edb.SCHEME_SSP3, 0.005, fix_entropy=True)
    b.load(f0)
    b.step(steps)
    F_b = b.read(real=True)
    srv = edb.Server(hbm_budget_bytes=4e9, scheme=edb.SCHEME_SSP3, dt=0.005, fix_entropy=True)
    ids = [srv.submit(N, 1.0, R, steps, f0[i], want_result=True) for i in range(3)]
    srv.run()
    for i, rid in enumerate(ids):
        F, _ = srv.result(rid)
        assert rel_l2(F, F_b[i]) <= 1e-12


def test_served_bkw_accuracy(edb):
    """BKW requests (Maxwell molecules, N = 24, L = 7, RK4 dt = 0.01, 50
    steps) served beside other traffic: L-inf <= 1e-6 against the exact BKW
    solution."""
    from entropydecreaseboltzmann_gb300 import data

    N, R, dt, steps = 24, 7.0, 0.01, 50
    t0 = [5.5, 6.5, 7.5]
    srv = edb.Server(hbm_budget_bytes=12e9, scheme=edb.SCHEME_RK4, dt=dt)
    ids = [srv.submit(N, 0.0, R, steps, data.bkw_grid(N, R, t), want_result=True) for t in t0]
    for j in range(6):
        srv.submit(16, 1.0, 6.0, 30, data.maxwellian_mixture_batch(1, 16, 6.0, seed=j)[0])
    srv.run()
    for t, rid in zip(t0, ids):
        F, _ = srv.result(rid)
        err = float(np.max(np.abs(F - data.bkw_grid(N, R, t + steps * dt))))
        assert err <= 1e-6, err
    assert edb.device_status() == 0


def test_continuous_admission_and_budget(edb):
    """A request arriving while a long one runs is admitted at the next step
    boundary (it does not wait for the long one to finish); with a budget that
    holds only a few slots every request still completes."""
    from entropydecreaseboltzmann_gb300 import data

    N, R = 12, 6.0
    f = data.maxwellian_mixture_batch(1, N, R, seed=3)[0]
    srv = edb.Server(hbm_budget_bytes=4e9, scheme=edb.SCHEME_RK4, dt=0.01)
    srv.prepare(N, 0.0, R)
    long_id = srv.submit(N, 0.0, R, 400, f)
    late_id = srv.submit(N, 0.0, R, 5, f, arrival_s=0.05)
    srv.run()
    a, b = srv.info(long_id), srv.info(late_id)
    assert b["t_admit"] < a["t_done"] and b["t_done"] < a["t_done"]
    assert b["t_admit"] - b["t_arrival"] < 0.5 * (a["t_done"] - a["t_admit"])
    st = srv.stats()
    assert st["completed"] == 2 and st["tts_p50_s"] <= st["tts_p99_s"]
    srv.close()
    # a budget of one table (the FP32 pair table: N (N/2 + 1) N^4 x 4 B =
    # 7.0 MB), its transfer staging (64 x N^3 x 40 B = 4.4 MB) and about 29
    # slots (N^3 x 248 B each: RK4 stages plus 8 chunk partial sums), so the 70
    # requests are served in waves
    srv = edb.Server(hbm_budget_bytes=2.4e7, scheme=edb.SCHEME_RK4, dt=0.01)
    for j in range(70):
        srv.submit(N, 0.0, R, 3, f)
    srv.run()
    st = srv.stats()
    assert st["completed"] == 70
    assert st["hbm_bytes_peak"] <= 2.4e7
    srv.close()
    # a request that can never fit is refused at submission
    srv = edb.Server(hbm_budget_bytes=1.0e6, scheme=edb.SCHEME_RK4, dt=0.01)
    with pytest.raises(edb.EdbError) as ei:
        srv.submit(N, 0.0, R, 3, f)
    assert ei.value.status == 2  # EDB_ENOMEM
    srv.close()


def test_conservative_serving(edb):
    """Conservative mode through the server: moments of each served solve
    kept to 1e-10 relative."""
    from entropydecreaseboltzmann_gb300 import data

    N, R = 12, 6.0
    f0 = data.maxwellian_mixture_batch(4, N, R, seed=31)
    srv = edb.Server(hbm_budget_bytes=4e9, scheme=edb.SCHEME_SSP3, dt=0.005, fix_entropy=True,
                     conserve=True)
    ids = [srv.submit(N, 1.0, R, 25 + 5 * i, f0[i], want_result=True) for i in range(4)]
    srv.run()
    h = 2 * R / N
    x = -R + h * np.arange(N)
    X, Y, Z = [a.reshape(-1) for a in np.meshgrid(x, x, x, indexing="ij")]
    phi = np.stack([np.ones_like(X), X, Y, Z, X * X + Y * Y + Z * Z])
    for i, rid in enumerate(ids):
        F, _ = srv.result(rid)
        m, m0 = phi @ F * h ** 3, phi @ f0[i] * h ** 3
        sc = np.array([m0[0], *(3 * [np.sqrt(m0[0] * m0[4])]), m0[4]])
        assert np.max(np.abs(m - m0) / sc) <= 1e-10


def test_uneven_batch_small(edb):
    """The uneven-batch workload at reduced size: 4 solves per N in
    {16, 24, 32} with gamma drawn from {0, 0.5, 1} (up to 9 tables, the
    non-integer gamma through quadrature), SSP3 with the moment-preserving
    fix, 3-8 steps each; every request completes."""
    from entropydecreaseboltzmann_gb300 import serving

    reqs = serving.uneven_requests(4, seed=7, steps=(3, 8))
    srv = edb.Server(hbm_budget_bytes=40e9, scheme=edb.SCHEME_SSP3, dt=0.005, fix_entropy=True,
                     conserve=True)
    st, _ = serving.run(srv, reqs, 0.005)
    assert st["completed"] == len(reqs) == 12
    assert 3 <= st["groups"] <= 9
    assert edb.device_status() == 0
    srv.close()


def test_background_loop_serves_concurrent_clients(edb):
    """edb_server_start: two client threads submit while the loop runs (arrival
    = now); every result equals the same solve run alone (bit-identical), and a
    request submitted after the others finished is still served."""
    import threading
    import time

    from entropydecreaseboltzmann_gb300 import data

    R, steps = 6.0, 12
    specs = [(12 if j % 2 else 16, float(j % 3 == 0), 4 + (j % 5)) for j in range(10)]
    inits = [data.maxwellian_mixture_batch(1, n, R, seed=500 + j)[0]
             for j, (n, _, _) in enumerate(specs)]
    # each request alone, through run()
    alone = []
    for (n, g, k), f in zip(specs, inits):
        s1 = edb.Server(hbm_budget_bytes=4e9, scheme=edb.SCHEME_RK4, dt=0.01)
        rid = s1.submit(n, g, R, steps + k, f, want_result=True)
        s1.run()
        alone.append(s1.result(rid)[0])
        s1.close()
    srv = edb.Server(hbm_budget_bytes=4e9, scheme=edb.SCHEME_RK4, dt=0.01)
    srv.start()
    ids = {}
    lock = threading.Lock()

    def client(part):
        for j in range(part, len(specs), 2):
            n, g, k = specs[j]
            rid = srv.submit(n, g, R, steps + k, inits[j], want_result=True)
            with lock:
                ids[j] = rid
            time.sleep(0.005)

    ths = [threading.Thread(target=client, args=(p,)) for p in (0, 1)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    for j in range(len(specs)):
        srv.wait(ids[j], 120.0)
        F, _ = srv.result(ids[j])
        assert np.array_equal(F, alone[j]), j
    # the loop idles, then takes new work
    late = srv.submit(12, 0.0, R, 3, inits[1], want_result=True)
    srv.wait(late, 60.0)
    assert srv.info(late)["state"] == 2
    srv.stop()
    st = srv.stats()
    assert st["completed"] == len(specs) + 1 and st["refused"] == 0
    srv.close()


def test_failure_paths_free_their_slots(edb):
    """Failures are handled on the host and free what they held; nothing on
    the device faults:
    * initial data with a NaN is refused at submit (EDB_EINVAL) and never
      queued;
    * a queued request that is cancelled never runs (EDB_ECANCELED from wait);
    * a running request that is cancelled is retired at the end of its step
      in flight: its slot is freed and the group's live count drops to 0;
    * a solve whose state overflows (initial data of 1e300 per cell) is
      reported as failed (EDB_ENONFINITE) and its slot freed;
    * the loop keeps serving: a request submitted afterwards completes and
      equals the same solve alone."""
    import time

    from entropydecreaseboltzmann_gb300 import data

    N, R = 12, 6.0
    f = data.maxwellian_mixture_batch(1, N, R, seed=21)[0]
    bad = f.copy()
    bad[7] = np.nan
    srv = edb.Server(hbm_budget_bytes=8e9, scheme=edb.SCHEME_RK4, dt=0.01)
    srv.prepare(N, 0.0, R)
    with pytest.raises(edb.EdbError) as e:
        srv.submit(N, 0.0, R, 5, bad)
    assert e.value.status == 1
    assert srv.stats()["submitted"] == 0

    srv.start()
    try:
        # cancelled while queued: arrives far in the future, never runs
        late = srv.submit(N, 0.0, R, 5, f, arrival_s=1e6)
        srv.cancel(late)
        with pytest.raises(edb.EdbError) as e:
            srv.wait(late, timeout_s=30)
        assert e.value.status == 8
        # cancelled while running
        long_id = srv.submit(N, 0.0, R, 10 ** 6, f)
        t0 = time.time()
        while srv.info(long_id)["state"] != 1:
            assert time.time() - t0 < 30
            time.sleep(0.01)
        srv.cancel(long_id)
        with pytest.raises(edb.EdbError) as e:
            srv.wait(long_id, timeout_s=30)
        assert e.value.status == 8
        # a state that overflows
        boom = srv.submit(N, 0.0, R, 3, np.full(N ** 3, 1e300))
        with pytest.raises(edb.EdbError) as e:
            srv.wait(boom, timeout_s=30)
        assert e.value.status == 9
        assert srv.info(boom)["state"] == 5
        # still serving
        ok = srv.submit(N, 0.0, R, 5, f, want_result=True)
        srv.wait(ok, timeout_s=60)
    finally:
        srv.stop()
    st = srv.stats()
    assert (st["cancelled"], st["failed"], st["completed"], st["live"], st["queued"]) == (2, 1, 1, 0, 0)
    F_ok, _ = srv.result(ok)
    srv.close()
    alone = edb.Server(hbm_budget_bytes=8e9, scheme=edb.SCHEME_RK4, dt=0.01)
    rid = alone.submit(N, 0.0, R, 5, f, want_result=True)
    alone.run()
    F_alone, _ = alone.result(rid)
    alone.close()
    assert rel_l2(F_ok, F_alone) <= 1e-12
