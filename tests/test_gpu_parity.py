"""GPU parity of the CUDA path against the oracle and the reference's golden vectors.

Tolerances
  FP64 calQ vs the reference QCalculator: relative L2 over modes <= 1e-12.
  genB vs the oracle's restatement of QCalculator::genB: max |dB| <= 1e-13 max|B|
    (only the last bits of CUDA's and glibc's sin/cos differ).
  FFT vs the oracle / numpy: <= 1e-13 relative to max |x|.
  Integrators vs the reference's runs: relative L2 of Fhat and F <= 1e-11;
    entropies <= 1e-11 relative.
  Batched FP32 calQ vs the FP64 oracle: relative L2 <= 5e-6.  Rounding the
    inputs (f-hat, B) to FP32 alone costs 4e-7 at N=24; FP32 accumulation of
    terms that cancel (gain minus loss) adds 1-3e-6 (a CPU emulation of the
    kernel's exact operation order reproduces the measured 2.2e-6).  In real
    space that is ~1e-8, two orders below the BKW target; the end-to-end
    criterion is test_batch_bkw_linf (L-inf <= 1e-6 against BKW).
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


@pytest.mark.parametrize("N,alpha,filt", [(N, a, f) for N in range(3, 10) for a, f in ((0, 1), (1, 0))])
def test_calQ_fp64_matches_reference_golden(edb, golden, N, alpha, filt):
    tag = f"N{N}_a{alpha}_f{filt}"
    q = edb.QCalculator(N, alpha, filter=bool(filt))
    q.genB()
    fin = golden[f"calq_in_{tag}"]
    Q = q.calQ(None, fin)
    assert rel_l2(Q, golden[f"calq_out_{tag}"]) <= 1e-12


@pytest.mark.parametrize("N", [5, 6, 8, 9])
@pytest.mark.parametrize("mode", [INDEX_REFERENCE, INDEX_ALIASED])
@pytest.mark.parametrize("gamma,filt", [(0.0, True), (1.0, False), (0.5, False), (0.5, True)])
def test_genB_matches_oracle(edb, oracle, N, mode, gamma, filt):
    """gamma 0 and 1: the reference's closed forms; gamma 0.5: the published
    integral by the same composite Gauss-Legendre rule on both sides."""
    q = edb.QCalculator(N, int(gamma), gamma=gamma, L=6.0, filter=filt, index_mode=mode)
    q.genB()
    B = q.B()
    Bo = oracle.genB(N, gamma, 6.0, filt, mode)
    assert np.max(np.abs(B - Bo)) <= 1e-13 * np.max(np.abs(Bo))


@pytest.mark.parametrize("N", [15, 16, 17])
def test_calQ_fp64_reference_mode_larger_N(edb, oracle, N):
    rng = np.random.default_rng(N)
    fin = rng.integers(0, 10, N ** 3) + 1j * rng.integers(0, 10, N ** 3)
    q = edb.QCalculator(N, 0)
    q.genB()
    Bo = oracle.genB(N, 0.0, R_REFERENCE, True, INDEX_REFERENCE)
    Qo = oracle.calQ(N, Bo, fin, INDEX_REFERENCE)
    assert rel_l2(q.calQ(None, fin), Qo) <= 1e-12
    # the same table fed from the oracle isolates the sum from genB
    q.set_B(Bo)
    assert rel_l2(q.calQ(None, fin), Qo) <= 1e-13


@pytest.mark.parametrize("N,L", [(16, 6.0), (17, 6.0)])
def test_calQ_fp64_aliased_bkw(edb, oracle, N, L):
    from entropydecreaseboltzmann_gb300 import data

    f = data.bkw_grid(N, L, 5.5)
    fhat = np.fft.fftn(f.reshape(N, N, N)).reshape(-1)
    q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    Bo = oracle.genB(N, 0.0, L, False, INDEX_ALIASED)
    Qo = oracle.calQ(N, Bo, fhat, INDEX_ALIASED)
    assert rel_l2(q.calQ(None, fhat), Qo) <= 1e-12


# radix-4/2 stages, odd-prime stages (3, 5, 7), primes taken whole (17), and
# N = 64 (the 131 KB shared-memory tile of the FP64 pass)
@pytest.mark.parametrize("N", [2, 3, 5, 6, 8, 12, 16, 17, 21, 24, 25, 32, 64])
def test_fft3d_matches_oracle(edb, oracle, N):
    rng = np.random.default_rng(N)
    x = rng.standard_normal(N ** 3) + 1j * rng.standard_normal(N ** 3)
    f = edb.fft3d()
    X = np.empty_like(x)
    f.fft(N, N, N, x, X)
    Xo = oracle.fft3d(N, x)
    assert np.max(np.abs(X - Xo)) <= 1e-13 * np.max(np.abs(Xo))
    y = np.empty_like(x)
    f.ifft(N, N, N, y, X)
    assert np.max(np.abs(y - oracle.fft3d(N, Xo, inverse=True))) <= 1e-13 * np.max(np.abs(x))


@pytest.mark.parametrize("N", [2, 3, 5, 6, 8, 12, 16, 17, 21, 24, 25, 32, 64])
def test_fft3d_double_float_matches_oracle(edb, oracle, N):
    """The double-float passes (FP64 data, hi + lo float arithmetic; the batch
    and the server use them): max error <= 1e-13 of max |X|, forward and
    inverse, over a batch of three cubes."""
    import torch

    rng = np.random.default_rng(300 + N)
    x = rng.standard_normal((3, N ** 3)) + 1j * rng.standard_normal((3, N ** 3))
    d = torch.from_numpy(x).cuda()
    X = torch.empty_like(d)
    edb.fft3d.device(N, 3, d, X, inverse=False, fp32=edb.fft3d.DOUBLE_FLOAT)
    y = torch.empty_like(d)
    edb.fft3d.device(N, 3, X, y, inverse=True, fp32=edb.fft3d.DOUBLE_FLOAT)
    torch.cuda.synchronize()
    X, y = X.cpu().numpy(), y.cpu().numpy()
    for c in range(3):
        Xo = oracle.fft3d(N, x[c])
        assert np.max(np.abs(X[c] - Xo)) <= 1e-13 * np.max(np.abs(Xo))
        yo = oracle.fft3d(N, X[c], inverse=True)
        assert np.max(np.abs(y[c] - yo)) <= 1e-13 * np.max(np.abs(yo))
        assert np.max(np.abs(y[c] - x[c])) <= 1e-13 * np.max(np.abs(x[c]))


@pytest.mark.parametrize("Nt", [10, 101, 1000])
def test_entropyfix_matches_reference(edb, golden, Nt):
    """Inputs of CalQ/testEntropyFix.cpp.  There the aim H(f2) equals H of the
    mean state, the minimum of H over the blend, so the bisection root sits
    where dH/dbeta -> 0 and round-off may move the accepted beta: entropies
    must agree to 1e-12, the fixed state must satisfy FixSol's contract and
    stay within 1e-6 of the reference's."""
    f1 = np.arange(Nt, dtype=np.float64)
    f2 = np.empty(Nt)
    f2[: Nt // 2] = np.floor((Nt - 1.0) / 2.0)
    f2[Nt // 2:] = np.ceil((Nt - 1.0) / 2.0)
    ef = edb.EntropyFix(Nt)
    e1 = ef.EntropyCal(f1)
    e2 = ef.EntropyCal(f2)
    g = f1.copy()
    ef.FixSol(g, e2)
    e3 = ef.EntropyCal(g)
    ref = golden[f"efix_{Nt}"]
    np.testing.assert_allclose([e1, e2, ef.average], ref[[0, 1, 3]], rtol=1e-12, atol=0)
    np.testing.assert_allclose(e3, ref[2], rtol=1e-9)
    assert e3 <= e2 + 1e-9 * abs(e2)
    ref_g = golden[f"efix_fixed_{Nt}"]
    assert np.max(np.abs(g - ref_g)) <= 1e-6 * np.max(np.abs(ref_g))
    # the result is a blend (1-beta) f + beta mean(f)
    beta = 1.0 - (g[-1] - g[0]) / (f1[-1] - f1[0])
    np.testing.assert_allclose(g, (1 - beta) * f1 + beta * np.mean(f1), rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("Nt", [64, 4096])
def test_entropyfix_well_conditioned_matches_reference(edb, golden, Nt):
    f = 1.0 + 0.5 * np.sin(np.arange(Nt) * 0.37) ** 2
    ref = golden[f"efixwc_{Nt}"]
    ef = edb.EntropyFix(Nt)
    e_f = ef.EntropyCal(f)
    np.testing.assert_allclose([e_f, ef.average], ref[[0, 4]], rtol=1e-13)
    g = f.copy()
    ef.FixSol(g, ref[2])
    ref_g = golden[f"efixwc_fixed_{Nt}"]
    assert np.max(np.abs(g - ref_g)) <= 1e-9 * np.max(np.abs(ref_g))
    np.testing.assert_allclose(ef.EntropyCal(g), ref[3], rtol=1e-10)


@pytest.mark.parametrize("scheme", ["FE", "CFE", "RK2", "SSP3", "RK4", "DUFORT"])
def test_integrators_match_reference(edb, golden, oracle, scheme):
    N = 6
    b = edb.BKW3D(N, R_REFERENCE)
    b.setFixEntropy(True)
    run = getattr(b, {"FE": "FEuler"}.get(scheme, scheme))
    if scheme in ("CFE", "DUFORT"):
        run(0.0, 0.05, 0.01, 2.0)
    else:
        run(0.0, 0.05, 0.01)
    assert rel_l2(b.Fhat, golden[f"run_{scheme}_Fhat"]) <= 1e-11
    assert rel_l2(b.F, golden[f"run_{scheme}_F"]) <= 1e-11
    _, _, raw, fixed = oracle.run(N, R_REFERENCE, scheme, 0.0, 0.05, 0.01, beta=2.0, fix=True)
    np.testing.assert_allclose(b.entropy_raw, raw, rtol=1e-11)
    np.testing.assert_allclose(b.entropy_fixed, fixed, rtol=1e-11)


def _batch_inputs(N, L, S, seed):
    from entropydecreaseboltzmann_gb300 import data

    F0, _, _ = data.bkw_bump_batch(S, N, L, seed)
    fh = np.fft.fftn(F0.reshape(S, N, N, N), axes=(1, 2, 3)).reshape(S, -1)
    return F0, fh


@pytest.mark.parametrize("N,L,S", [(3, 6.0, 2), (4, 6.0, 5), (5, 6.0, 3), (8, 6.0, 17),
                                   (16, 6.0, 37), (24, 7.0, 20)])
def test_calQ_batch_fp32_matches_fp64_oracle(edb, oracle, N, L, S):
    import torch

    _, fh = _batch_inputs(N, L, S, seed=7 + N)
    q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    fin = torch.from_numpy(fh.astype(np.complex64)).cuda()
    out = torch.empty_like(fin)
    q.calQ_batch_f32(S, fin, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    Bo = oracle.genB(N, 0.0, L, False, INDEX_ALIASED)
    for s in range(S):
        Qo = oracle.calQ(N, Bo, fh[s], INDEX_ALIASED)
        assert rel_l2(got[s], Qo) <= 5e-6, s


def test_batch_result_same_alone_and_in_the_mix(edb):
    """Each solve of the batched kernel is independent of its batch mates."""
    import torch

    N, L, S = 8, 6.0, 21
    _, fh = _batch_inputs(N, L, S, seed=3)
    q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    fin = torch.from_numpy(fh.astype(np.complex64)).cuda()
    mix = torch.empty_like(fin)
    q.calQ_batch_f32(S, fin, mix)
    for s in (0, 5, 20):
        one = torch.empty_like(fin[s:s + 1])
        q.calQ_batch_f32(1, fin[s:s + 1].contiguous(), one)
        torch.cuda.synchronize()
        assert torch.equal(one[0], mix[s])


@pytest.mark.parametrize("N,L,chunks", [(8, 6.0, 4), (9, 6.0, 3), (16, 6.0, 8), (24, 7.0, 8)])
def test_calQ_batch_variants_and_chunks(edb, oracle, N, L, chunks):
    """Every variant (16- and 4-solve groups, 8 or 4 outputs per thread,
    registers / shared memory for the compensated sums, plain or solve-pair
    input layout; N = 9 takes the plain-load path) gives bit-identical
    results for a given chunk count (S = 11: the last pair has one solve),
    a solve alone equals the same solve in a batch, and chunked and unchunked
    results meet the FP32 tolerance (relative L2 <= 5e-6) against the FP64
    oracle."""
    import torch

    S = 11
    _, fh = _batch_inputs(N, L, S, seed=40 + N)
    q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    fin = torch.from_numpy(fh.astype(np.complex64)).cuda()
    part = torch.empty(chunks * S * N ** 3 * 4, dtype=torch.float32, device="cuda")
    res = {}
    for C in (1, chunks):
        for v in range(edb.lib.edb_qcalc_batch_variants()):
            out = torch.empty_like(fin)
            try:
                q.calQ_batch_f32_ex(S, v, C, part, fin, out)
            except edb.EdbError as e:  # unknown variant, or one that does not fit this N
                assert e.status == 1 and v > 0
                continue
            torch.cuda.synchronize()
            res[(C, v)] = out.cpu().numpy()
        for (c, v), r in res.items():
            if c == C:
                assert np.array_equal(r, res[(C, 0)]), v
        assert len([k for k in res if k[0] == C]) >= 6
        for v in (2, 7):
            one = torch.empty_like(fin[3:4])
            q.calQ_batch_f32_ex(1, v, C, part, fin[3:4].contiguous(), one)
            torch.cuda.synchronize()
            assert np.array_equal(one.cpu().numpy()[0], res[(C, 0)][3])
    Bo = oracle.genB(N, 0.0, L, False, INDEX_ALIASED)
    for s in (0, 7):
        Qo = oracle.calQ(N, Bo, fh[s], INDEX_ALIASED)
        for C in (1, chunks):
            assert rel_l2(res[(C, 0)][s], Qo) <= 5e-6
    assert edb.device_status() == 0


def test_device_calQ_matches_host_calQ(edb):
    import torch

    N = 9
    rng = np.random.default_rng(5)
    fin = rng.standard_normal(N ** 3) + 1j * rng.standard_normal(N ** 3)
    q = edb.QCalculator(N, 0)
    q.genB()
    Qh = q.calQ(None, fin)
    d_in = torch.from_numpy(fin).cuda()
    d_out = torch.empty_like(d_in)
    q.calQ_device(d_in, d_out)
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy(), Qh)


def test_batch_bkw_linf(edb):
    """North-star criterion of the FP32 path: RK4 (dt = 0.01) on BKW initial
    data at N = 24, L = 7 for 50 steps; L-inf error against the exact BKW
    solution <= 1e-6 at the end (the FP64 discretisation floor at this size
    is 9.6e-7 in dQ/dt; the error is stated for every output time)."""
    from entropydecreaseboltzmann_gb300 import data

    N, L, S, dt = 24, 7.0, 8, 0.01
    t0 = np.linspace(5.5, 8.0, S)
    q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    b = edb.BatchSolver(q, S, L, edb.SCHEME_RK4, dt)
    b.load(np.stack([data.bkw_grid(N, L, t) for t in t0]))
    errs = []
    for step in range(1, 51):
        b.step(1)
        if step % 10 == 0:
            f = b.read(real=True)
            exact = np.stack([data.bkw_grid(N, L, t + step * dt) for t in t0])
            errs.append(float(np.max(np.abs(f - exact))))
    assert edb.device_status() == 0
    assert max(errs) <= 1e-6, errs


@pytest.mark.parametrize("N,mode", [(9, INDEX_REFERENCE), (16, INDEX_REFERENCE), (17, INDEX_ALIASED),
                                    (24, INDEX_ALIASED)])
def test_fp64_emulated_kernel_matches_native_and_oracle(edb, oracle, N, mode):
    """The double-float FP64 kernel (default) and the native-FP64 kernel
    against the oracle: relative L2 <= 1e-12 on random integer data and on
    BKW data.  Up to N = 17 against the oracle's full sum; at N = 24 (whose
    table the oracle would hold as 1.5 GB) against the oracle's direct
    evaluation of the aliased sum at 128 sampled modes."""
    from entropydecreaseboltzmann_gb300 import data

    rng = np.random.default_rng(1000 + N)
    q = edb.QCalculator(N, 0, L=7.0, filter=(mode == INDEX_REFERENCE), index_mode=mode)
    q.genB()
    f_bkw = np.fft.fftn(data.bkw_grid(N, 7.0, 6.0).reshape(N, N, N)).reshape(-1)
    f_int = rng.integers(0, 10, N ** 3) + 1j * rng.integers(0, 10, N ** 3)
    Bo = oracle.genB(N, 0.0, 7.0, mode == INDEX_REFERENCE, mode) if N <= 17 else None
    modes = rng.choice(N ** 3, 128, replace=False)
    tuned = q.fp64_shape()
    for fin in (f_int, f_bkw):
        q.set_fp64_kernel(0)
        Qe = q.calQ(None, fin)
        q.set_fp64_kernel(1)
        Qn = q.calQ(None, fin)
        if Bo is not None:
            Qo = oracle.calQ(N, Bo, fin, mode)
            assert rel_l2(Qe, Qo) <= 1e-12
            assert rel_l2(Qn, Qo) <= 1e-12
        else:
            assert mode == INDEX_ALIASED
            Qd = oracle.direct_modes(N, fin, modes, gamma=0.0, R=7.0, filter=False)
            assert rel_l2(Qe[modes], Qd) <= 1e-12
            assert rel_l2(Qn[modes], Qd) <= 1e-12
        # every launch shape of the double-float kernel (CTA size, register
        # cap, rows per ring slot, and either rule for the l-line chunks)
        # meets the same bound
        q.set_fp64_kernel(0)
        for shp in range(edb.lib.edb_qcalc_fp64_shapes()):
            q.fp64_shape(shp)
            Qs = q.calQ(None, fin)
            if Bo is not None:
                assert rel_l2(Qs, Qo) <= 1e-12, shp
            else:
                assert rel_l2(Qs[modes], Qd) <= 1e-12, shp
        q.fp64_shape(tuned)
    with pytest.raises(edb.EdbError):
        q.fp64_shape(edb.lib.edb_qcalc_fp64_shapes())


def test_funF_and_filtering_on_device_match_reference_golden(edb, golden):
    """QCalculator.funF / .filtering (device evaluation) against the
    reference's values: <= 1e-13 of the largest value (CUDA's and glibc's
    sin/cos differ in the last bits, which cancellation near xi = eta
    magnifies relative to small values, as for genB)."""
    grid, vals = golden["funF_grid"], golden["funF_val"]
    for alpha in (0, 1):
        sel = grid[:, 0] == alpha
        q = edb.QCalculator(5, alpha)
        got = q.funF(grid[sel, 1], grid[sel, 2])
        want = vals[sel]
        assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))
    for N in sorted(set(int(n) for n in golden["filtering"][:, 0])):
        rows = golden["filtering"][golden["filtering"][:, 0] == N]
        q = edb.QCalculator(N, 0)
        got = q.filtering(rows[:, 1].astype(np.int32))
        assert np.max(np.abs(got - rows[:, 2])) <= 1e-13 * np.max(np.abs(rows[:, 2]))


@pytest.mark.parametrize("S", [1, 3, 11, 17])
def test_batch_load_read_round_trip(edb, oracle, S):
    """Load and read move the state in cube chunks on a second stream (S not a
    multiple of the chunk count, fewer solves than chunks): read(load(f)) = f
    to FFT round-off, into a caller's buffer too, and Fhat after load is the
    FP64 transform of each solve (<= 1e-13 against the oracle's DFT)."""
    N, L = 12, 6.0
    rng = np.random.default_rng(300 + S)
    f = rng.standard_normal((S, N ** 3))
    q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    b = edb.BatchSolver(q, S, L, edb.SCHEME_RK4, 0.01)
    b.load(f)
    back, fh = b.read(real=True, fhat=True)
    assert np.max(np.abs(back - f)) <= 1e-13 * np.max(np.abs(f))
    for s in range(S):
        want = oracle.fft3d(N, f[s].astype(np.complex128))
        assert np.max(np.abs(fh[s] - want)) <= 1e-13 * np.max(np.abs(want))
    out = np.empty((S, N ** 3))
    b.read(real=True, out=out)
    assert np.array_equal(out, back)
