"""The input layer (fall3d_gb300.inputs): the .inp keyword reader with the
reference's number decoding, the .grn and .src files, the TGSD and Suzuki
source generators, and a scenario built from files that runs through the
oracle."""
import math

import numpy as np
import pytest

import oracle_lib as O
from fall3d_gb300 import inputs as I
from fall3d_gb300 import synth

INP = """!  a control file in the layout of the FALL3D 7.0 input files
 TIME_UTC
   YEAR = 2010
   MONTH = 04
   BEGIN_METEO_DATA_(HOURS_AFTER_00) = 0
   TIME_STEP_METEO_DATA_(MIN) = 60
   ERUPTION_START_(HOURS_AFTER_00) = 0 3.5
   RUN_END_(HOURS_AFTER_00) = 0.5   ! half an hour
 GRID
   COORDINATES = LON-LAT
   LON_LAT
      LONMIN = 14.0
      LONMAX = 15.5
      LATMIN = 37.0
      LATMAX = 38.0
   NX = 31
   NY = 21
   ZLAYER_(M)  FROM 0. TO 8000. INCREMENT 500.
 GRANULOMETRY
   DISTRIBUTION = BIGAUSSIAN
   NUMBER_OF_CLASSES = 6
   FI_MEAN = 2.5 4.0
   FI_DISP = 1.5 1.0
   FI_RANGE = -1 5
   DENSITY_RANGE = 1200 2300
   SPHERICITY_RANGE = 0.9 0.9
 SUZUKI_SOURCE
   HEIGHT_ABOVE_VENT_(M) = 6000.
   MASS_FLOW_RATE_(KGS)  = 1.5d6
   A = 4.
   L = 5.
"""


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_inp_reader(tmp_path):
    f = I.read_inp(_write(tmp_path, "run.inp", INP))
    assert f.integer("TIME_UTC", "YEAR") == [2010]
    assert f.real("TIME_UTC", "ERUPTION_START_(HOURS_AFTER_00)", 2) == [0.0, 3.5]
    assert f.char("GRID", "COORDINATES") == ["LON-LAT"]
    assert f.real("GRID", "LONMIN") == [14.0]
    z = f.real("GRID", "ZLAYER_(M)", 0)
    assert len(z) == 17 and z[0] == 0.0 and z[-1] == 8000.0
    assert f.npar("GRANULOMETRY", "FI_MEAN") == 2
    assert f.real("SUZUKI_SOURCE", "MASS_FLOW_RATE_(KGS)") == [1.5e6]
    with pytest.raises(KeyError):
        f.real("GRID", "NZ")
    with pytest.raises(ValueError):
        f.real("GRANULOMETRY", "FI_DISP", 3)


def test_number_decoding_follows_decode_f90():
    # digits accumulate as the reference's stof does: 0.3 is 3*(1/10),
    # one ulp above the correctly rounded 0.3
    assert I.stof("0.3") == 3 * (1.0 / 10.0)
    assert I.stof("0.3") != 0.3
    assert I.stof("1d3") == 1000.0
    assert I.stof("1.25D2") == 125.0
    assert I.stof("-2.") == -2.0
    assert I.stof("+7") == 7.0
    assert I.stof("1.5E-3") == (1.0 + 5 * 0.1) / 1000.0
    words, params = I.sdecode("   FI_RANGE = -1 5 ! comment")
    assert words == ["FI_RANGE", "!", "comment"] and params == [-1.0, 5.0]


def test_grn_round_trip_and_setfrac(tmp_path):
    g = I.setfrac(6, -1.0, 5.0, 1200.0, 2300.0, 0.9, 0.9, [2.5, 4.0], [1.5, 1.0])
    # the two Gaussians' weights are the binary32 literals 0.98 and 0.02
    assert abs(sum(g["fc"]) - (float(np.float32(0.98)) + float(np.float32(0.02)))) < 1e-6
    assert np.all(np.diff(g["diam_mm"]) < 0) and g["diam_mm"][0] == 2.0
    p = str(tmp_path / "run.grn")
    I.write_grn(p, g["diam_mm"], g["rhop"], g["sphe"], g["fc"])
    r = I.read_grn(p)
    assert r["nc"] == 6
    assert np.allclose(r["diam_mm"], g["diam_mm"], atol=5e-7)
    assert np.allclose(r["rhop"], g["rhop"], atol=0.05)
    assert np.allclose(r["fc"], g["fc"], rtol=1e-8)


def test_fer_is_the_trapezoidal_normal_cdf():
    # the reference's loop stops as soon as the accumulated t2 reaches |x|:
    # depending on the rounding of that sum the last slab of width |x|/10000
    # is integrated or not, so fer is the normal CDF or short of it by the
    # slab
    for x in (-2.0, -0.3, 0.0, 0.7, 3.0):
        exact = 0.5 * (1.0 + math.erf(x / math.sqrt(2.0)))
        slab = abs(x) / 10000.0 * math.exp(-x * x / 2.0) / math.sqrt(2.0 * math.pi)
        d = abs(I.fer(x) - exact)
        assert d < 1e-7 or abs(d - slab) < 1e-7 + 1e-3 * slab


def test_suzuki_getsrc_and_src_round_trip(tmp_path):
    nx, ny = 11, 9
    xorigr, yorigr, dx, dy = 14.0, 37.0, 0.05, 0.05
    zmodel = np.linspace(0.0, 8000.0, 17)
    fc = np.array([0.5, 0.3, 0.2])
    X0, Y0 = xorigr + 5 * dx, yorigr + 4 * dy  # the vent on node (6, 5)
    xp, yp, zp, mp = I.solvesuzuki(50, 6000.0, 4.0, 5.0, 1e6, fc, X0, Y0, 0.0, 0.0)
    src = I.getsrc(xp, yp, zp, mp, xorigr, yorigr, dx, dy, nx, ny, zmodel, np.zeros((ny, nx)), 0.0)
    assert abs(src.sum() - 1e6) < 1e-6 * 1e6
    # all on the vent's column, as synth's node-centred restatement puts it
    col = src[:, 5, 4, :]
    assert abs(col.sum() - src.sum()) < 1e-6
    zrel, mplum = synth.suzuki_column(50, 6000.0, 4.0, 5.0, 1e6, fc)
    ref = synth.distribute_column(zrel, mplum, zmodel, len(zmodel))
    assert np.allclose(col.T, ref, rtol=1e-12, atol=1e-9)
    rec = I.src_interval(src, 0, 3600, xorigr, yorigr, dx, dy, zmodel)
    p = str(tmp_path / "run.src")
    I.write_src(p, [rec, dict(t1=3600, t2=999999, x=[], y=[], z=[], i=[], j=[], k=[],
                              rates=np.zeros((0, 3)))])
    r = I.read_src(p)
    assert list(r["nsou"]) == [len(rec["i"]), 0]
    assert list(r["isrc"]) == rec["i"] and list(r["ksrc"]) == rec["k"]
    n = len(rec["i"])
    got = r["tmrat"].reshape(3, n).T
    assert np.allclose(got, rec["rates"], rtol=1e-8)


def test_scenario_from_files_runs_in_the_oracle(tmp_path):
    inp = _write(tmp_path, "run.inp", INP)
    f = I.read_inp(inp)
    g = I.setfrac(6, -1.0, 5.0, 1200.0, 2300.0, 0.9, 0.9, [2.5, 4.0], [1.5, 1.0])
    grn = str(tmp_path / "run.grn")
    I.write_grn(grn, g["diam_mm"], g["rhop"], g["sphe"], g["fc"])
    nx, ny = f.integer("GRID", "NX")[0], f.integer("GRID", "NY")[0]
    zmodel = np.array(f.real("GRID", "ZLAYER_(M)", 0))
    dx = (15.5 - 14.0) / (nx - 1)
    dy = (38.0 - 37.0) / (ny - 1)
    xp, yp, zp, mp = I.solvesuzuki(100, 6000.0, 4.0, 5.0, 1.5e6, g["fc"], 14.0 + 15 * dx, 37.0 + 10 * dy, 0.0, 0.0)
    src = I.getsrc(xp, yp, zp, mp, 14.0, 37.0, dx, dy, nx, ny, zmodel, np.zeros((ny, nx)), 0.0)
    rec = I.src_interval(src, 0, 86400, 14.0, 37.0, dx, dy, zmodel)
    srcp = str(tmp_path / "run.src")
    I.write_src(srcp, [rec])
    s = I.scenario_from_files(inp, grn, srcp, seed=3, max_snapshots=2)
    assert s.grid["nx"] == nx and s.grid["nz"] == len(zmodel) and s.grid["nc"] == 6
    o = O.OracleCtx(s, nthreads=4)
    log = o.run(max_steps=4)
    assert o.state()["iiter"] == 4 and log["massvol"][-1] > 0.0


def test_setpsi_matches_the_reference():
    """inputs.setpsi (with get_gama's bisection) against the reference's own
    Sources/setpsi.f90 (tests/golden/setpsi.npz, made by
    tests/golden/make_setpsi_golden.py), bit for bit, for the four settling
    models."""
    import os

    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "setpsi.npz"))
    for modv in (1, 2, 3, 4):
        psi = I.setpsi(modv, d["sphe"], d["diam"])
        assert np.array_equal(psi.view(np.uint64), d[f"psi{modv}"].view(np.uint64)), modv


def test_short_or_garbled_files_are_read_errors(tmp_path):
    """A .grn or .src file cut short, or with a word that is not a number,
    is the readers' read error (libMaster/get_granulometry_value.f90:79-82,
    get_source_value.f90:80-85), with the reference's message, not a Python
    index error."""
    g = I.setfrac(4, 0.0, 3.0, 1200.0, 2300.0, 0.9, 0.9, [1.5], [1.0])
    p = str(tmp_path / "run.grn")
    I.write_grn(p, g["diam_mm"], g["rhop"], g["sphe"], g["fc"])
    text = open(p).read()
    for bad in (text[: len(text) // 2], text.replace(text.split()[3], "x.y", 1), "", "3\n"):
        open(p, "w").write(bad)
        with pytest.raises(ValueError, match="error reading the granulometry file"):
            I.read_grn(p)
    rates = np.array([[1.0, 2.0], [3.0, 4.0]])
    rec = dict(t1=0, t2=3600, x=[14.0, 14.1], y=[37.0, 37.1], z=[100.0, 200.0], i=[1, 2], j=[1, 2],
               k=[1, 2], rates=rates)
    rec2 = dict(rec, t1=3600, t2=7200)
    q = str(tmp_path / "run.src")
    I.write_src(q, [rec, rec2])
    text = open(q).read()
    assert I.read_src(q)["nsou"].tolist() == [2, 2]
    lines = text.splitlines(keepends=True)
    open(q, "w").write("".join(lines[:-1]))  # the second interval's last source line missing
    with pytest.raises(ValueError, match=r"error reading the source file at time\s+3600"):
        I.read_src(q)
    open(q, "w").write(text.replace(text.split()[1], "abc", 1))
    with pytest.raises(ValueError, match="error reading the source file"):
        I.read_src(q)
