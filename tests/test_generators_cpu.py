"""The pre-processing generators of the input layer (fall3d_gb300/inputs.py)
against the reference's own utilities, bit for bit: SetTgsd's setfrac.f90
(diameters, densities, sphericities and Gaussian / bi-Gaussian fractions with
the trapezoidal normal CDF fer), SetSrc's solvesuzuki.f90 (the Suzuki
column) and getsrc.f90 (the column spread over the nodes and levels).  The
fixture tests/golden/generators.npz was made from the translated utilities by
tests/golden/make_generators_golden.py."""
import os

import numpy as np

from fall3d_gb300 import inputs

GOLD = os.path.join(os.path.dirname(__file__), "golden", "generators.npz")
TGSD = [(6, -1.0, 4.0, 1000.0, 2500.0, 0.9, 0.9, [1.5], [1.5]),
        (16, -2.0, 6.0, 800.0, 2700.0, 0.6, 0.95, [1.0, 4.5], [1.2, 0.8]),
        (9, 0.0, 8.0, 1200.0, 1200.0, 0.7, 1.0, [3.3], [2.1])]
SUZUKI = [(100, 8000.0, 4.0, 5.0, 1.0e6, 0.37, 0.41, 1500.0, 0.0),
          (50, 15000.0, 8.0, 1.5, 3.2e7, 0.52, 0.23, 900.0, 120.0)]
ZMODEL = np.array([0.0, 100.0, 300.0, 700.0, 1300.0, 2000.0, 3000.0, 4500.0, 6500.0, 9000.0, 12000.0, 16000.0,
                   21000.0])
NX, NY = 20, 16


def same(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_setfrac_matches_the_reference():
    d = np.load(GOLD)
    for k, case in enumerate(TGSD):
        r = inputs.setfrac(*case)
        assert same(r["fc"], d[f"tgsd{k}_fc"]), k
        assert same(r["diam_mm"], d[f"tgsd{k}_diam"]), k
        assert same(r["rhop"], d[f"tgsd{k}_rhop"]), k
        assert same(r["sphe"], d[f"tgsd{k}_sphe"]), k


def test_solvesuzuki_and_getsrc_match_the_reference():
    d = np.load(GOLD)
    topg_ref = d["topg"]  # (nx+1, ny+1) node elevations of the reference's layout
    for k, (ns, H, A, L, M0, X0, Y0, Z0, dZ0) in enumerate(SUZUKI):
        fc = d[f"tgsd{k}_fc"]
        xp, yp, zp, mp = inputs.solvesuzuki(ns, H, A, L, M0, fc, X0, Y0, Z0, dZ0)
        assert same(xp, d[f"src{k}_xplum"]) and same(yp, d[f"src{k}_yplum"]), k
        assert same(zp, d[f"src{k}_zplum"]), k
        assert same(mp, d[f"src{k}_mplum"]), k
        src = inputs.getsrc(xp, yp, zp, mp, 0.0, 0.0, 0.05, 0.05, NX, NY, ZMODEL,
                            np.ascontiguousarray(topg_ref[:NX, :NY].T), dZ0)
        want = d[f"src{k}_src"][:, :NX, :NY, :len(ZMODEL)]
        assert same(src, want), k
        assert src.sum() > 0.5 * M0
