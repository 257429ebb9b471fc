"""The CPU oracle pinned against the reference's own outputs.

Golden vectors come from the reference headers compiled unmodified
(tests/golden/make_golden.py).  Every comparison here is bit-exact: the oracle
restates the reference's arithmetic operation by operation.
"""
import numpy as np
import pytest

from oracle.oracle import INDEX_ALIASED, INDEX_REFERENCE, R_REFERENCE, EntropyFixOracle

CASES = [(N, a, f) for N in range(3, 10) for a, f in ((0, 1), (1, 0))]


@pytest.mark.parametrize("N,alpha,filt", CASES)
def test_calQ_matches_reference_golden(oracle, golden, N, alpha, filt):
    tag = f"N{N}_a{alpha}_f{filt}"
    B = oracle.genB(N, alpha, R_REFERENCE, bool(filt), INDEX_REFERENCE)
    nq = N ** 3
    if f"B_{tag}" in golden:
        assert np.array_equal(B, golden[f"B_{tag}"])
    else:
        for i, r in enumerate(golden[f"Brows_idx_{tag}"]):
            assert np.array_equal(B[r * nq:(r + 1) * nq], golden[f"Brows_{tag}"][i])
        w = np.cos(np.arange(nq * nq) * 0.001)
        s = golden[f"Bsum_{tag}"]
        assert np.dot(B, w) == pytest.approx(s[0], rel=1e-13, abs=1e-13 * s[1])
        assert np.sum(np.abs(B)) == pytest.approx(s[1], rel=1e-14)
    Q = oracle.calQ(N, B, golden[f"calq_in_{tag}"], INDEX_REFERENCE)
    assert np.array_equal(Q, golden[f"calq_out_{tag}"])


@pytest.mark.parametrize("N", [3, 5, 7, 9])
def test_aliased_equals_reference_for_odd_N(oracle, golden, N):
    tag = f"N{N}_a0_f1"
    B = oracle.genB(N, 0.0, R_REFERENCE, True, INDEX_ALIASED)
    Q = oracle.calQ(N, B, golden[f"calq_in_{tag}"], INDEX_ALIASED)
    assert np.array_equal(Q, golden[f"calq_out_{tag}"])


@pytest.mark.parametrize("N", [4, 5, 6, 8])
def test_direct_evaluator_equals_aliased_table(oracle, N):
    rng = np.random.default_rng(N)
    fin = rng.standard_normal(N ** 3) + 1j * rng.standard_normal(N ** 3)
    for gamma, filt in ((0.0, True), (1.0, False)):
        B = oracle.genB(N, gamma, 6.0, filt, INDEX_ALIASED)
        Qa = oracle.calQ(N, B, fin, INDEX_ALIASED)
        Qd = oracle.direct(N, fin, gamma, 6.0, filt)
        assert np.array_equal(Qa, Qd)


def test_funF_and_filtering_match_reference(oracle, golden):
    for (a, x, e), v in zip(golden["funF_grid"], golden["funF_val"]):
        assert oracle.funF(int(a), x, e) == v
    for N, b, v in golden["filtering"]:
        assert oracle.filtering(int(N), int(b)) == v


def test_funF_readme_special_values(oracle):
    # ReadMe.md:62-67
    assert oracle.funF(0, 0.0, 0.0) == pytest.approx(1 / 3)
    assert oracle.funF(1, 0.0, 0.0) == pytest.approx(1 / 4)
    x = 0.7
    assert oracle.funF(0, x, 0.0) == pytest.approx((-x * np.cos(x) + np.sin(x)) / x ** 3)
    assert oracle.funF(0, x, x) == pytest.approx((x - np.cos(x) * np.sin(x)) / (2 * x ** 3))


@pytest.mark.parametrize("gamma", [0.0, 1.0])
def test_quadrature_matches_closed_forms(oracle, gamma):
    lam = 2.0 / (3.0 + np.sqrt(2.0)) * np.pi
    for a in (0, 1, 3, 12, 48, 300, 3072):
        for b in (0, 2, 3, 12, 110, 2883):
            xi, eta = np.sqrt(a) * lam, np.sqrt(b) * lam
            assert abs(oracle.funF_quad(gamma, xi, eta) - oracle.funF(int(gamma), xi, eta)) < 5e-15


@pytest.mark.parametrize("Nt", [10, 101, 1000])
def test_entropyfix_matches_reference(oracle, golden, Nt):
    f1 = np.arange(Nt, dtype=np.float64)
    f2 = np.empty(Nt)
    f2[: Nt // 2] = np.floor((Nt - 1.0) / 2.0)
    f2[Nt // 2:] = np.ceil((Nt - 1.0) / 2.0)
    ef = EntropyFixOracle(oracle, Nt)
    e1 = ef.EntropyCal(f1)
    e2 = ef.EntropyCal(f2)
    g = f1.copy()
    ef.FixSol(g, e2)
    e3 = ef.EntropyCal(g)
    ref = golden[f"efix_{Nt}"]
    assert [e1, e2, e3, ef.average] == list(ref)
    assert np.array_equal(g, golden[f"efix_fixed_{Nt}"])


@pytest.mark.parametrize("Nt", [64, 4096])
def test_entropyfix_well_conditioned_matches_reference(oracle, golden, Nt):
    f = 1.0 + 0.5 * np.sin(np.arange(Nt) * 0.37) ** 2
    ref = golden[f"efixwc_{Nt}"]
    ef = EntropyFixOracle(oracle, Nt)
    assert ef.EntropyCal(f) == ref[0]
    g = f.copy()
    ef.FixSol(g, ref[2])
    assert np.array_equal(g, golden[f"efixwc_fixed_{Nt}"])
    assert ef.EntropyCal(g) == ref[3]


@pytest.mark.parametrize("N", [5, 6, 8])
def test_initial_data_and_entropy(oracle, golden, N):
    F0 = oracle.initial_sinusoid(N, R_REFERENCE)
    assert np.array_equal(F0, golden[f"init_{N}"])
    assert oracle.calentropy(N, R_REFERENCE, F0) == golden[f"entropy_init_{N}"][0]


@pytest.mark.parametrize("scheme", ["FE", "CFE", "RK2", "SSP3", "RK4", "DUFORT"])
def test_integrators_match_reference(oracle, golden, scheme):
    from oracle.oracle import parse_entropy_log

    Fhat, F, raw, fixed = oracle.run(6, R_REFERENCE, scheme, 0.0, 0.05, 0.01, beta=2.0, fix=True)
    assert np.array_equal(Fhat, golden[f"run_{scheme}_Fhat"])
    assert np.array_equal(F, golden[f"run_{scheme}_F"])
    # every entropy the oracle records (before and after the fix) is printed by
    # the reference with 8 decimals (BKW.h:228-241, 431-444, 501-514)
    log = str(golden[f"run_{scheme}_log"])
    for v in list(raw) + list(fixed):
        assert f"{v:.8f}" in log, (scheme, v)


def test_fft_conventions(oracle):
    N = 6
    rng = np.random.default_rng(3)
    x = rng.standard_normal(N ** 3) + 1j * rng.standard_normal(N ** 3)
    X = oracle.fft3d(N, x)
    np.testing.assert_allclose(X, np.fft.fftn(x.reshape(N, N, N)).reshape(-1), rtol=0, atol=1e-12)
    xi = oracle.fft3d(N, X, inverse=True)
    np.testing.assert_allclose(xi, x, rtol=0, atol=1e-13)


def test_reference_library_agrees_with_restatement(oracle, reference):
    """Only where the reference sources exist: live cross-check at N=7, 8."""
    rng = np.random.default_rng(11)
    for N in (7, 8):
        q = reference.qcalc(N, 0, True)
        fin = rng.standard_normal(N ** 3) + 1j * rng.standard_normal(N ** 3)
        B = oracle.genB(N, 0.0, R_REFERENCE, True, INDEX_REFERENCE)
        assert np.array_equal(q.B(), B)
        assert np.array_equal(q.calQ(fin), oracle.calQ(N, B, fin, INDEX_REFERENCE))


def test_reference_output_files_fixture(reference, tmp_path):
    """The committed output-file fixtures are exactly what the compiled
    reference writes for FEuler at N = 6 (F.dat and outV1Direction)."""
    import os

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        reference.fe_files(6, 6.62132, 0.0, 0.05, 0.01, True, "slice.dat")
    finally:
        os.chdir(cwd)
    for got, want in (("F.dat", "ref_FE_N6_F.dat"), ("slice.dat", "ref_FE_N6_slice.dat")):
        assert (tmp_path / got).read_bytes() == open(os.path.join(here, want), "rb").read()


# ---- the workloads' sizes (tests/golden/reference_golden_configs.npz)

@pytest.fixture(scope="module")
def cfg():
    import os

    return np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_golden_configs.npz"))


@pytest.mark.parametrize("tag", ["sin", "bkw"])
def test_config1_rk4_oracle_matches_reference(oracle, cfg, tag):
    """The testBKW3D case on RK4 (N = 16, [-6, 6]^3, dt = 0.01): the oracle's
    restated step sequence from the same initial data gives the reference's
    bits after 10 steps (the checkpoint both fixtures hold)."""
    checks = list(cfg[f"cfg1_{tag}_checks"])
    i = checks.index(10)
    Fh, F, raw, fixed = oracle.run(16, 6.0, "RK4", 0.0, 9.5 * 0.01, 0.01, fix=True,
                                   F0=cfg[f"cfg1_{tag}_F0"])
    assert np.array_equal(Fh, cfg[f"cfg1_{tag}_Fhat"][i])
    np.testing.assert_array_equal(raw, cfg[f"cfg1_{tag}_ent_raw"][:10])
    np.testing.assert_array_equal(fixed, cfg[f"cfg1_{tag}_ent_fixed"][:10])
    if tag == "sin":
        assert np.array_equal(F, cfg["cfg1_sin_F"])


@pytest.mark.parametrize("N", [15, 16, 17])
def test_ssp3_fix_oracle_matches_reference(oracle, cfg, N):
    """SSP3 with the fix rule, 10 steps of dt = 0.005 (the fix acts on steps
    2-10 at N = 16): bit-identical final Fhat, F and entropy traces."""
    Fh, F, raw, fixed = oracle.run(N, R_REFERENCE, "SSP3", 0.0, 9.5 * 0.005, 0.005, fix=True,
                                   F0=cfg[f"ssp3_N{N}_F0"])
    assert np.array_equal(Fh, cfg[f"ssp3_N{N}_Fhat"])
    assert np.array_equal(F, cfg[f"ssp3_N{N}_F"])
    np.testing.assert_array_equal(raw, cfg[f"ssp3_N{N}_ent_raw"])
    np.testing.assert_array_equal(fixed, cfg[f"ssp3_N{N}_ent_fixed"])
    if N == 16:
        assert np.count_nonzero(raw != fixed) >= 5  # the fix acted


def test_calQ_N25_direct_modes_match_reference(oracle, cfg):
    """calQ at N = 25 (odd: the reference's loops are the aliased sum) against
    the oracle's direct evaluation at 64 modes, relative L2 <= 1e-13 (the two
    sums run in different orders)."""
    N = 25
    fin = cfg["calq_in_N25_a1_f0"]
    want = cfg["calq_out_N25_a1_f0"]
    k = np.random.default_rng(25).choice(N ** 3, 64, replace=False)
    got = oracle.direct_modes(N, fin, k, gamma=1.0, R=R_REFERENCE, filter=False)
    assert np.linalg.norm(got - want[k]) <= 1e-13 * np.linalg.norm(want[k])
