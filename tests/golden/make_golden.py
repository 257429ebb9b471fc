"""Generates tests/golden/reference_golden.npz from the compiled reference.

Run where the reference sources exist:  python tests/golden/make_golden.py
It builds oracle/_ref/libedbref.so (make -C oracle ref) from the reference's
own CalQ headers and records, for fixed seeds:

* QCalculator::calQ outputs (CalQ/QCalculator.h:231-257) for N = 3..9,
  Maxwell + filter and hard-sphere without filter, on integer-valued complex
  inputs in [0, 10) like CalQ/test.cpp:19-21;
* the B table (QCalculator.h:158-229): in full for N = 3, 4 and three full
  rows plus a weighted checksum for N = 5..9;
* funF (:76-106) on a grid of (xi, eta) and filtering (:67-74) for N = 3..33;
* EntropyFix (EntropyFix.h) on the inputs of CalQ/testEntropyFix.cpp:22-38;
* the sinusoid initial data (BKW.h:96-138) and calEntropy (:140-152);
* full BKW3D integrator runs (FE, CFE, RK2, SSP3, RK4, DUFORT) at N = 6,
  T = 0.05, dt = 0.01, beta = 2: final Fhat, final F and the printed log;
* the reference's output files of that FEuler run, as text beside the .npz:
  ref_FE_N6_F.dat (BKW.h:217-249) and ref_FE_N6_slice.dat (outV1Direction,
  BKW.h:163-180).

The FFTs inside those runs come from the in-repo FFTW-API shim, because FFTW
is not installed here; its conventions are FFTW's documented ones.

A second file, tests/golden/reference_golden_configs.npz, holds the cases at
the workloads' sizes (``--configs`` regenerates only it):

* the testBKW3D case on RK4 (CalQ/BKW.h:452-519): N = 16 on [-6, 6]^3,
  dt = 0.01, 100 steps, the reference's QCalculator(N0, 0).  Once from the
  BKW profile at t0 = 5.5 (K = 1 - exp(-t0/6), CalQ/testfft.cpp:11-16):
  Fhat after steps 1, 10, 50 and 100, F after step 100, and every step's
  entropy before / after the fix rule.  Once more from the reference's own
  initial data (setInitialValue's live sinusoid branch, BKW.h:96-138) for
  10 steps (after step 10 that run turns most modes into NaN under the
  even-N loops); it is checked here to be bit-identical to the reference's
  own BKW3D::RK4;
* SSP3 with the fix rule (BKW.h:387-449), 10 steps of dt = 0.005, on
  [-6.62132, 6.62132]^3: N = 16 from the sinusoid (the fix acts on steps
  2-10) and N = 15, 17 from a seeded two-Maxwellian mixture;
* QCalculator::calQ at N = 24 (Maxwell, filter on) and N = 25 (hard sphere,
  filter off) on integer-valued inputs.
Runs from data other than the sinusoid go through oracle/ref_wrap.cpp's
edbref_run_from, which drives the reference's own objects.
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference, build_oracle, _ptr  # noqa: E402

R = 6.62132


def _data_module():
    # the initial-data helpers, loaded by path (importing the package would
    # load its CUDA library)
    import importlib.util

    path = os.path.join(ROOT, "entropydecreaseboltzmann_gb300", "data.py")
    spec = importlib.util.spec_from_file_location("edb_data", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


CFG1_CHECKS = [1, 10, 50, 100]
CFG1_SIN_CHECKS = [1, 5, 10]


def configs(ref):
    data = _data_module()
    out = {}
    # ---- the testBKW3D case on RK4: N = 16, R = 6, dt = 0.01, 100 steps
    N, Rb, dt = 16, 6.0, 0.01
    # the sinusoid under the even-N loops turns most modes into NaN between
    # steps 10 and 19, so that run stops at step 10
    for tag, F0, checks in (("sin", ref.initial(N, Rb), CFG1_SIN_CHECKS),
                            ("bkw", data.bkw_grid(N, Rb, 5.5), CFG1_CHECKS)):
        TEnd = (checks[-1] - 0.5) * dt  # `do { t += dt } while (t < TEnd)`: checks[-1] steps
        Fh, F, raw, fixed = ref.run_from(N, Rb, "RK4", F0, 0.0, TEnd, dt, checks)
        assert np.all(np.isfinite(Fh)) and np.all(np.isfinite(F))
        out[f"cfg1_{tag}_F0"] = np.asarray(F0, dtype=np.complex128)
        out[f"cfg1_{tag}_Fhat"] = Fh
        out[f"cfg1_{tag}_F"] = F[-1]
        out[f"cfg1_{tag}_ent_raw"] = raw
        out[f"cfg1_{tag}_ent_fixed"] = fixed
        out[f"cfg1_{tag}_checks"] = np.array(checks)
        if tag == "sin":  # the reference's own driver gives the same bits
            Fl, Fll, _ = ref.run(N, Rb, "RK4", 0.0, TEnd, dt, fix=True)
            assert np.array_equal(Fl, Fh[-1]) and np.array_equal(Fll, F[-1])
    # ---- SSP3 with the fix rule, N = 15 / 16 / 17, 10 steps of dt = 0.005
    dt3 = 0.005
    for N in (15, 16, 17):
        F0 = ref.initial(N, R) if N == 16 else data.two_maxwellians(N, R, 100 + N)
        Fh, F, raw, fixed = ref.run_from(N, R, "SSP3", F0, 0.0, 9.5 * dt3, dt3, [10])
        out[f"ssp3_N{N}_F0"] = np.asarray(F0, dtype=np.complex128)
        out[f"ssp3_N{N}_Fhat"] = Fh[0]
        out[f"ssp3_N{N}_F"] = F[0]
        out[f"ssp3_N{N}_ent_raw"] = raw
        out[f"ssp3_N{N}_ent_fixed"] = fixed
    # ---- calQ at the workloads' N (REFERENCE loops; odd N = the aliased sum)
    rng = np.random.default_rng(20211024)
    for N, alpha, filt in ((24, 0, True), (25, 1, False)):
        tag = f"N{N}_a{alpha}_f{int(filt)}"
        q = ref.qcalc(N, alpha, filt)
        fin = rng.integers(0, 10, N ** 3) + 1j * rng.integers(0, 10, N ** 3)
        out[f"calq_in_{tag}"] = fin
        out[f"calq_out_{tag}"] = q.calQ(fin)
        del q
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden_configs.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes,", len(out), "arrays")


def main():
    build_oracle(ref=True)
    ref = Reference()
    out = {}
    rng = np.random.default_rng(20210413)
    # ---- calQ and B
    for N in range(3, 10):
        for alpha, filt in ((0, True), (1, False)):
            tag = f"N{N}_a{alpha}_f{int(filt)}"
            q = ref.qcalc(N, alpha, filt)
            fin = rng.integers(0, 10, N ** 3) + 1j * rng.integers(0, 10, N ** 3)
            out[f"calq_in_{tag}"] = fin
            out[f"calq_out_{tag}"] = q.calQ(fin)
            B = q.B()
            nq = N ** 3
            if N <= 4:
                out[f"B_{tag}"] = B
            else:
                rows = [0, nq // 2, nq - 1]
                out[f"Brows_idx_{tag}"] = np.array(rows)
                out[f"Brows_{tag}"] = np.stack([B[r * nq:(r + 1) * nq] for r in rows])
                w = np.cos(np.arange(nq * nq) * 0.001)
                out[f"Bsum_{tag}"] = np.array([np.dot(B, w), np.sum(np.abs(B))])
            del q
    # ---- funF / filtering
    xs = np.array([0.0, 1e-11, 0.3, 0.4534, 0.9068, 1.7, 3.2, 7.5, 19.0, 41.3])
    grid = np.array([[a, x, e] for a in (0, 1) for x in xs for e in xs])
    out["funF_grid"] = grid
    out["funF_val"] = np.array([ref.funF(int(a), x, e) for a, x, e in grid])
    fil = []
    for N in range(3, 34):
        for b in range(-(N // 2) - 1, N // 2 + 2):
            fil.append((N, b, ref.filtering(N, b)))
    out["filtering"] = np.array(fil)
    # ---- EntropyFix (testEntropyFix.cpp inputs)
    for Nt in (10, 101, 1000):
        f1 = np.arange(Nt, dtype=np.float64)
        f2 = np.empty(Nt)
        f2[: Nt // 2] = np.floor((Nt - 1.0) / 2.0)
        f2[Nt // 2:] = np.ceil((Nt - 1.0) / 2.0)
        h = ref.L.edbref_efix_new(Nt, 1.0e-10)
        e1 = ref.L.edbref_efix_entropy(h, Nt, _ptr(f1))
        e2 = ref.L.edbref_efix_entropy(h, Nt, _ptr(f2))
        g = f1.copy()
        ref.L.edbref_efix_fixsol(h, Nt, _ptr(g), e2)
        e3 = ref.L.edbref_efix_entropy(h, Nt, _ptr(g))
        out[f"efix_{Nt}"] = np.array([e1, e2, e3, ref.L.edbref_efix_average(h)])
        out[f"efix_fixed_{Nt}"] = g
        ref.L.edbref_efix_free(h)
    # ---- EntropyFix, well-conditioned: aim halfway between H(f) and H(mean f),
    # so the bisection root has a nonzero slope
    for Nt in (64, 4096):
        f = 1.0 + 0.5 * np.sin(np.arange(Nt) * 0.37) ** 2
        h = ref.L.edbref_efix_new(Nt, 1.0e-10)
        e_f = ref.L.edbref_efix_entropy(h, Nt, _ptr(f))
        avg = ref.L.edbref_efix_average(h)
        fbar = np.full(Nt, avg)
        e_bar = ref.L.edbref_efix_entropy(h, Nt, _ptr(fbar))
        aim = 0.5 * (e_f + e_bar)
        g = f.copy()
        ref.L.edbref_efix_fixsol(h, Nt, _ptr(g), aim)
        e_g = ref.L.edbref_efix_entropy(h, Nt, _ptr(g))
        out[f"efixwc_{Nt}"] = np.array([e_f, e_bar, aim, e_g, avg])
        out[f"efixwc_fixed_{Nt}"] = g
        ref.L.edbref_efix_free(h)
    # ---- initial data / entropy
    for N in (5, 6, 8):
        F0 = ref.initial(N, R)
        out[f"init_{N}"] = F0
        out[f"entropy_init_{N}"] = np.array([ref.calentropy(N, R, F0)])
    # ---- integrators (FEuler writes F.dat into the working directory)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as td:
        os.chdir(td)
        try:
            for scheme in ("FE", "CFE", "RK2", "SSP3", "RK4", "DUFORT"):
                Fhat, F, log = ref.run(6, R, scheme, 0.0, 0.05, 0.01, beta=2.0, fix=True)
                out[f"run_{scheme}_Fhat"] = Fhat
                out[f"run_{scheme}_F"] = F
                out[f"run_{scheme}_log"] = np.array(log)
            # the output files of FEuler + outV1Direction, byte for byte
            ref.fe_files(6, R, 0.0, 0.05, 0.01, True, "slice.dat")
            here = os.path.dirname(os.path.abspath(__file__))
            for src, dst in (("F.dat", "ref_FE_N6_F.dat"), ("slice.dat", "ref_FE_N6_slice.dat")):
                with open(src, "rb") as fi, open(os.path.join(here, dst), "wb") as fo:
                    fo.write(fi.read())
        finally:
            os.chdir(cwd)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    if "--configs" in sys.argv:
        build_oracle(ref=True)
        configs(Reference())
    else:
        main()
        configs(Reference())
