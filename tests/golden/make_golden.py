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
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference, build_oracle, _ptr  # noqa: E402

R = 6.62132


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
    main()
