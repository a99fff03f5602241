"""The meteorological database (DBS) layer (fall3d_gb300/dbs.py) against the
reference's own get_dbs_value_plane.f90 (tests/golden/dbs_plane.npz, made by
tests/golden/make_dbs_golden.py from the translated routine).

The database is written to a file in the SetDbs schema (classic netCDF with
64-bit offsets), read back and every query of the fixture is compared bit
for bit: the time interval (the last interval holding the time), the end
time, and the vertical interpolation (clamped to the first and last level,
the last pair of levels around a height that lies on a level)."""
import numpy as np
import pytest

from fall3d_gb300 import dbs, synth

pytest.importorskip("scipy")
GOLD = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "dbs_plane.npz")


def _write(tmp_path, d):
    met = {"U": d["U"], "RHO": d["RHO"], "PBLH": d["PBLH"], "LDU": d["LDU"], "times": d["times"]}
    # the other 3-D fields are not queried; write copies so the file has the full schema
    for k in ("V", "W", "T", "TP", "P", "QV"):
        met[k] = d["U"]
    for k in ("UST", "RMOL", "ZNT", "PRATE"):
        met[k] = d["PBLH"]
    path = tmp_path / "dbs.nc"
    dbs.write_dbs(path, met, d["alt"])
    return path


def test_planes_match_the_reference_routine(tmp_path):
    d = np.load(GOLD)
    path = _write(tmp_path, d)
    ds = dbs._open(path)
    try:
        assert ds.version_byte == 2  # NF90_64BIT_OFFSET
        assert int(ds.NT) == len(d["times"]) and int(ds.NZ) == len(d["alt"])
        for q in range(len(d["q_word"])):
            word, t, z = str(d["q_word"][q]), int(d["q_time"][q]), float(d["q_z"][q])
            plane, endsec = dbs.get_dbs_value_plane(ds, t, word, z)
            assert endsec == int(d["endsec"][q]), (word, t, z)
            want = d["planes"][q]
            assert np.array_equal(plane.view(np.uint64), want.view(np.uint64)), (word, t, z)
    finally:
        ds.close()


def test_errors_of_the_reference():
    d = np.load(GOLD)
    with pytest.raises(dbs.DBSError, match="not in the database interval"):
        dbs.dbs_interval(d["times"], int(d["times"][0]) - 1)
    with pytest.raises(dbs.DBSError, match="not in the database interval"):
        dbs.dbs_interval(d["times"], int(d["times"][-1]) + 1)
    assert dbs.dbs_interval(d["times"], int(d["times"][-1])) == (len(d["times"]) - 1, int(d["times"][-1]))


def test_read_dbs_is_reamet_on_every_record(tmp_path):
    """A synthetic scenario's met written on its own levels and read back on
    the model levels gives the scenario's met series (binary32 values), the
    reference's defaults where PBLH / ZNT / PRATE are missing."""
    s = synth.make_scenario("tiny", seed=4, max_snapshots=3)
    g = s.grid
    alt = np.asarray(g["zlayer"], np.float32)
    met = {k: s.met[k] for k in ("u", "v", "w", "t", "tp", "rho", "ust", "rmol", "ldu")}
    met["times"] = s.met["times"]
    path = tmp_path / "tiny.nc"
    dbs.write_dbs(path, met, alt)
    out, warn = dbs.read_dbs(path, g["zlayer"], wetdep=True)
    assert np.array_equal(out["times"], s.met["times"])
    for k in ("u", "v", "w", "t", "tp", "rho"):
        assert np.array_equal(out[k], np.asarray(s.met[k], np.float32).astype(np.float64)), k
    assert np.all(out["pblh"] == 1500.0) and np.all(out["znt"] == 0.1) and np.all(out["prate"] == 0.0)
    assert len(warn) == 3 * len(s.met["times"])
    assert np.array_equal(out["ldu"], np.asarray(s.met["ldu"], np.float32).astype(np.float64))


def test_read_dbs_interpolates_between_levels(tmp_path):
    """Model levels between the DBS levels take the linear interpolation of
    get_dbs_value_plane.f90:140-160 (binary64 from binary32 data)."""
    nt, nz, ny, nx = 2, 4, 3, 5
    alt = np.array([0.0, 1000.0, 2000.0, 4000.0], np.float32)
    lin = lambda z: 2.0 + 0.003 * z
    u = np.broadcast_to(lin(alt.astype(np.float64))[None, :, None, None], (nt, nz, ny, nx)).astype(np.float32)
    met = {k: u for k in ("U", "V", "W", "T", "TP", "RHO")}
    met.update({k: np.ones((nt, ny, nx), np.float32) for k in ("UST", "RMOL", "PBLH", "ZNT", "PRATE")})
    met["times"] = np.array([0, 3600], np.int32)
    path = tmp_path / "lin.nc"
    dbs.write_dbs(path, met, alt)
    zl = np.array([0.0, 500.0, 1500.0, 3000.0, 5000.0])
    out, warn = dbs.read_dbs(path, zl)
    assert not warn
    want = np.array([lin(0.0), lin(500.0), lin(1500.0), lin(3000.0), lin(4000.0)])
    assert np.allclose(out["u"][0, :, 0, 0], want, rtol=1e-6)


def test_get_par_abl_matches_the_reference():
    """fall3d_gb300.dbs.get_par_abl against the reference's own
    Utilities/SetDbs/get_par_ABL.f90 (tests/golden/setdbs_abl.npz, made by
    tests/golden/make_setdbs_golden.py from the translated routine), bit for
    bit, over stable and unstable columns, calm air and equal temperatures."""
    d = np.load(GOLD.replace("dbs_plane.npz", "setdbs_abl.npz"))
    n = len(d["z0"])
    assert n >= 400
    ri_signs = set()
    for i in range(n):
        args = [float(d[k][i]) for k in ("z0", "z1", "tz0", "tz1", "pz0", "pz1", "u", "v")]
        ust, rmo = dbs.get_par_abl(*args)
        assert np.float64(ust).view(np.uint64) == d["ustar"][i].view(np.uint64), i
        assert np.float64(rmo).view(np.uint64) == d["rmonin"][i].view(np.uint64), i
        ri_signs.add(args[3] * (1.01e5 / args[5]) ** 0.285 > args[2] * (1.01e5 / args[4]) ** 0.285)
    assert ri_signs == {True, False}  # both branches exercised


def test_debug_dbs_is_read_back(tmp_path):
    """A DBS of SetDbs's DEBUG model (read_DEBUG_data.f90) written and read on
    the model levels: constant fields, the columns' ust from get_par_abl,
    RMOL 0 (SetDbs leaves it at its initial value), PBLH 1000 m."""
    zl = np.array([0.0, 250.0, 700.0, 1500.0, 3000.0])
    met = dbs.debug_dbs(6, 5, zl, [0, 3600])
    path = tmp_path / "debug.nc"
    dbs.write_dbs(path, met, zl.astype(np.float32))
    out, warn = dbs.read_dbs(path, zl, wetdep=True)
    assert not warn
    assert np.all(out["u"] == 10.0) and np.all(out["v"] == 0.0) and np.all(out["t"] == 273.0)
    assert np.all(out["rho"] == 1.0) and np.all(out["pblh"] == 1000.0) and np.all(out["rmol"] == 0.0)
    ust, _ = dbs.get_par_abl(1.0, 250.0, 273.0, 273.0, 1e5, 1e5, 10.0, 0.0)
    assert np.all(out["ust"] == np.float64(np.float32(ust)))
