"""The reference's restart file (fall3d_gb300/restart.py, Sources/wrirst.f90
and rearst.f90): written and read back, the contents are the binary32 values
of c with its halo and of cload = cdry + cwet, the erupted and outflow masses
exactly, and a file of another grid or domain is refused as rearst.f90
refuses it."""
import numpy as np
import pytest

from fall3d_gb300 import restart

pytest.importorskip("scipy")


def _state(nx=7, ny=5, nz=4, nc=3, seed=2):
    rng = np.random.default_rng(seed)
    c = rng.random((nc, nz + 2, ny + 2, nx + 2)) * 1e-3
    cdry = rng.random((nc + 1, ny, nx))
    cwet = rng.random((nc + 1, ny, nx)) * 0.1
    return c, cdry, cwet


def test_write_then_read(tmp_path):
    c, cdry, cwet = _state()
    nc, nz2, ny2, nx2 = c.shape
    bounds = (10.0, 10.6, 37.0, 37.4)
    p = tmp_path / "run.rst.nc"
    restart.write_reference_restart(p, c, cdry, cwet, 1.2345e9, 6.5e7, 0.0, 10800.0, bounds, date=(2015, 3, 8))
    r = restart.read_reference_restart(p, nx2 - 2, ny2 - 2, nz2 - 2, nc, bounds)
    assert np.array_equal(r["c"], c.astype(np.float32).astype(np.float64))
    assert np.array_equal(r["cload"], (cdry + cwet).astype(np.float32).astype(np.float64))
    assert r["erumass"] == 1.2345e9 and r["outmass"] == 6.5e7
    assert (r["run_start"], r["run_end"], r["date"]) == (0, 10800, (2015, 3, 8))
    from scipy.io import netcdf_file

    f = netcdf_file(p, "r", mmap=False)
    assert f.version_byte == 1 and set(f.variables) == {"CON", "LOAD"}
    assert f.variables["CON"].typecode() == "f" and f.variables["LOAD"].typecode() == "f"
    f.close()


def test_inconsistent_restart_is_refused(tmp_path):
    c, cdry, cwet = _state()
    nc, nz2, ny2, nx2 = c.shape
    bounds = (10.0, 10.6, 37.0, 37.4)
    p = tmp_path / "run.rst.nc"
    restart.write_reference_restart(p, c, cdry, cwet, 1.0, 0.0, 0.0, 3600.0, bounds)
    with pytest.raises(restart.RestartError, match="nz"):
        restart.read_reference_restart(p, nx2 - 2, ny2 - 2, nz2 - 1, nc, bounds)
    with pytest.raises(restart.RestartError, match="nc"):
        restart.read_reference_restart(p, nx2 - 2, ny2 - 2, nz2 - 2, nc + 1, bounds)
    with pytest.raises(restart.RestartError, match="latmax"):
        restart.read_reference_restart(p, nx2 - 2, ny2 - 2, nz2 - 2, nc, (10.0, 10.6, 37.0, 37.5))
