"""The reference's restart file, written and read beside the context's own
lossless checkpoint (f3d_ctx_save / f3d_ctx_restore).

FALL3D writes a restart at the end of a run (Sources/Fall3d.f90:133,
wrirst.f90) and a run with RESTART = yes reads it during its set-up
(setup.f90:116, rearst.f90).  The file is classic netCDF (NF90_CLOBBER) with
the dimensions nx, ny, nc, nc1 = nc+1, nx2 = nx+2, ny2 = ny+2, nz2 = nz+2, the
binary32 variables CON (the scaled concentration with its halo,
c(0:nx+1,0:ny+1,0:nz+1,nc)) and LOAD (the scaled ground load,
cload(nx,ny,0:nc) = cdry + cwet, endstep.f90:35,60), and the global attributes
TITLE, COORDINATES, YEAR, MONTH, DAY, RUN_START, RUN_END, ERUPTED_MASS,
OUT_MASS and the domain bounds (LONMIN.. or XMIN..) (wrirst.f90:28-207).

Reading (rearst.f90) checks nx, ny, nz, nc and the bounds against the run
and stops on a mismatch (:141-149), then sets c from CON, cload from LOAD
and the erupted and outflow masses from the attributes; cdry and cwet start
from zero and the drag-coefficient chain of setvset from its initial value,
as in the reference (its restart stores neither).  So a restarted run differs
from an uninterrupted one by the binary32 storage of c and by the deposit
history; ``fall3d_gb300.Context.save`` / ``restore`` is the lossless
alternative.
"""
from __future__ import annotations

import numpy as np


class RestartError(RuntimeError):
    """The reference's runend in rearst.f90."""


def write_reference_restart(path, c, cdry, cwet, erumass, outmass, beg_time, end_time, bounds,
                            coord_sys="LON-LAT", date=(2000, 1, 1)):
    """wrirst.f90: c (nc, nz+2, ny+2, nx+2) and cdry/cwet (nc+1, ny, nx) as a
    context's fields(); bounds = (lonmin, lonmax, latmin, latmax) or (xmin,
    xmax, ymin, ymax) for UTM."""
    from scipy.io import netcdf_file

    c = np.asarray(c)
    nc, nz2, ny2, nx2 = c.shape
    ny, nx = ny2 - 2, nx2 - 2
    f = netcdf_file(path, "w", version=1)  # NF90_CLOBBER: the classic format
    for name, n in (("nx", nx), ("ny", ny), ("nc", nc), ("nc1", nc + 1), ("nx2", nx2), ("ny2", ny2),
                    ("nz2", nz2)):
        f.createDimension(name, n)
    con = f.createVariable("CON", "f4", ("nc", "nz2", "ny2", "nx2"))
    load = f.createVariable("LOAD", "f4", ("nc1", "ny", "nx"))
    load.units, load.description = b"kg/m2", b"Scaled ground deposit load"
    con.units, con.description = b"gr/m3", b"Scaled concentration"
    f.TITLE = b"Fall3d 6.2 results"
    f.COORDINATES = coord_sys.encode()
    f.YEAR, f.MONTH, f.DAY = (np.int32(v) for v in date)
    f.RUN_START, f.RUN_END = np.int32(int(beg_time)), np.int32(int(end_time))
    f.ERUPTED_MASS, f.OUT_MASS = np.float64(erumass), np.float64(outmass)
    names = ("LONMIN", "LONMAX", "LATMIN", "LATMAX") if coord_sys == "LON-LAT" else ("XMIN", "XMAX", "YMIN", "YMAX")
    for n, v in zip(names, bounds):
        setattr(f, n, np.float64(v))
    con[:] = np.asarray(c, dtype=np.float32)
    load[:] = (np.asarray(cdry) + np.asarray(cwet)).astype(np.float32)  # cload = cdry + cwet
    f.close()


def read_reference_restart(path, nx, ny, nz, nc, bounds, coord_sys="LON-LAT"):
    """rearst.f90: checks the file against the run and returns c (binary64 of
    the file's binary32, (nc, nz+2, ny+2, nx+2)), cload (nc+1, ny, nx),
    erumass, outmass and the run window of the run that wrote it."""
    from scipy.io import netcdf_file

    f = netcdf_file(path, "r", mmap=False)
    try:
        dims = {k: int(v) for k, v in f.dimensions.items()}
        got = dict(nx=dims.get("nx"), ny=dims.get("ny"), nz=dims.get("nz2", 2) - 2, nc=dims.get("nc"))
        for k, want in (("nx", nx), ("ny", ny), ("nz", nz), ("nc", nc)):
            if got[k] != want:
                raise RestartError(f"restart inconsistency in {k}")
        names = ("LONMIN", "LONMAX", "LATMIN", "LATMAX") if coord_sys == "LON-LAT" else ("XMIN", "XMAX", "YMIN", "YMAX")
        for n, want in zip(names, bounds):
            if float(getattr(f, n)) != float(want):  # rearst.f90:146-149 compares exactly
                raise RestartError(f"restart inconsistency in {n.lower()}")
        c = np.array(f.variables["CON"][:], dtype=np.float64)
        cload = np.array(f.variables["LOAD"][:], dtype=np.float64)
        return dict(c=c, cload=cload, erumass=float(f.ERUPTED_MASS), outmass=float(f.OUT_MASS),
                    run_start=int(f.RUN_START), run_end=int(f.RUN_END),
                    date=(int(f.YEAR), int(f.MONTH), int(f.DAY)))
    finally:
        f.close()


def save_reference_restart(ctx, path, beg_time, end_time, bounds, coord_sys="LON-LAT", date=(2000, 1, 1)):
    """wrirst.f90 for a fall3d_gb300.Context at the end of its run."""
    f, st = ctx.fields(), ctx.state()
    write_reference_restart(path, f["c"], f["cdry"], f["cwet"], st["erumass"], st["outmass"], beg_time,
                            end_time, bounds, coord_sys, date)


def load_reference_restart(ctx, path, bounds, coord_sys="LON-LAT"):
    """setup.f90:116 / rearst.f90 into a fall3d_gb300.Context that has had its
    source and meteo updates: c, erumass and outmass from the file, cdry and
    cwet zero, the drag chain at its initial value.  Returns the file's
    contents (cload included: the reference replaces it by cdry + cwet at the
    first mass-budget step, endstep.f90:35)."""
    g = ctx.s.grid
    r = read_reference_restart(path, g["nx"], g["ny"], g["nz"], g["nc"], bounds, coord_sys)
    z = np.zeros((g["nc"] + 1, g["ny"], g["nx"]))
    ctx.upload_state(r["c"], z, z, r["erumass"], r["outmass"], 1.0)
    return r
