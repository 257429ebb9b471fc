"""The reference's BKW3D output files written by this build (F.dat rows of
FEuler, BKW.h:217-249; outV1Direction's slice, BKW.h:163-180), compared with
the compiled reference's files for the same run (N = 6, sinusoid initial
data, FEuler with the fix, T = 0.05, dt = 0.01).

Line structure and field counts must match exactly.  The printed values carry
6 (F.dat) or 8 (slice, fixed) digits; they must agree to the last printed
digit, up to one unit where the GPU's and the host's last bits straddle a
rounding boundary."""
import os

import numpy as np
import pytest

from oracle.oracle import R_REFERENCE

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _compare(got_path, want_path, abs_tol_of):
    got = open(got_path).read().split("\n")
    want = open(want_path).read().split("\n")
    assert len(got) == len(want)
    same = total = 0
    for g, w in zip(got, want):
        gf, wf = g.split("\t"), w.split("\t")
        assert len(gf) == len(wf)
        for a, b in zip(gf, wf):
            total += 1
            if a == b:
                same += 1
                continue
            x, y = float(a), float(b)  # numbers only may differ
            assert abs(x - y) <= abs_tol_of(b), (a, b)
    assert same >= 0.99 * total, (same, total)


def test_F_dat_and_slice_match_reference(tmp_path):
    import entropydecreaseboltzmann_gb300 as edb

    b = edb.BKW3D(6, R_REFERENCE, record_F=True)
    b.setFixEntropy(True)
    b.FEuler(0.0, 0.05, 0.01)
    assert b.F_history.shape == (b.nsteps, 216)
    assert np.array_equal(b.F_history[-1], b.F.real)
    b.write_F_dat(tmp_path / "F.dat")
    b.outV1Direction(tmp_path / "slice.dat")
    # %g with 6 significant digits: one unit in the sixth digit
    _compare(tmp_path / "F.dat", os.path.join(GOLD, "ref_FE_N6_F.dat"),
             lambda s: 1.01e-5 * max(abs(float(s)), 1e-300) + 1e-300)
    # fixed with 8 decimals: one unit in the eighth decimal
    _compare(tmp_path / "slice.dat", os.path.join(GOLD, "ref_FE_N6_slice.dat"),
             lambda s: 1.01e-8)
    assert edb.BKW3D.slice_filename(16, 0.01) == "N16.dt0.010000.dat"
