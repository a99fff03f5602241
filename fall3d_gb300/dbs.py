"""The meteorological database (DBS) of FALL3D: the netCDF file SetDbs writes
and the transport model reads, restated without the netCDF library.

* ``write_dbs`` writes a DBS in the schema of the reference's SetDbs utility
  (Utilities/SetDbs/write_DBS_grid.f90, write_DBS_data.f90, variable names of
  DBS_nc.f90): the classic format with 64-bit offsets (NF90_64BIT_OFFSET,
  write_DBS_grid.f90:27), dimensions lon/lat (or x/y for UTM), alt and time,
  binary32 fields and binary64 times, the global attributes NX, NY, NZ, NT,
  START_TIME, END_TIME, TIME_INCREMENT, COORDINATES, ...
* ``get_dbs_value_plane`` restates libMaster/get_dbs_value_plane.f90: the
  time interval of a time in seconds (:105-114, the last interval that
  holds it) and, for the 3-D variables, linear interpolation between the two
  DBS levels around a terrain-following height (:140-160), clamped to the
  first and last level.
* ``read_dbs`` is Sources/reamet.f90 for every snapshot of the file: the 3-D
  fields U, V, W, T, TP, P, RHO, QV on the model levels zlayer, and UST,
  PBLH, RMOL, ZNT, PRATE; a missing PBLH, ZNT or PRATE takes the reference's
  default (1500 m, 0.1 m, 0 mm/s, reamet.f90:96-145).  It returns the met
  series dictionary the context's f3d_run takes (f3d_met_series): PRATE stays
  in mm/s and vz(:,:,1) is not zeroed here, since the device's meteo update
  applies reamet.f90:146,153 itself.

* ``debug_dbs`` is SetDbs's DEBUG meteorological model
  (Utilities/SetDbs/read_DEBUG_data.f90, ``TYPE_DATA = debug``) with the
  friction velocity and Monin-Obukhov length of ``get_par_abl``
  (Utilities/SetDbs/get_par_ABL.f90): the fields a DBS made from it holds.

The file layer is scipy's implementation of the netCDF classic formats
(scipy.io.netcdf_file), which reads and writes the 64-bit-offset variant.
"""
from __future__ import annotations

import math

import numpy as np

# Utilities/SetDbs/DBS_nc.f90:22-62
VARS_2D_STATIC = ("XLON", "XLAT", "UTM_X", "UTM_Y", "TOPG", "LDU", "SOIL", "VEGFRA")
VARS_2D_TIME = ("PBLH", "UST", "SMOI", "RMOL", "ZNT", "SPD10", "L", "PRATE")
VARS_3D = ("U", "V", "W", "T", "TP", "P", "QV", "RHO")
# the dictionary of get_dbs_value_plane.f90:46-83: 0 static 2-D, 1 time-dependent 2-D, 2 3-D
VARCASE = {**{w: 0 for w in ("XLON", "XLAT", "UTM_X", "UTM_Y", "UTM_ZONE", "LDU", "SOIL", "VEGFRA", "TOPG")},
           **{w: 1 for w in ("PBLH", "UST", "SMOI", "RMOL", "ZNT", "SPD10", "PRATE", "L")},
           **{w: 2 for w in ("U", "V", "W", "T", "TP", "P", "QV", "RHO", "TV")}}


class DBSError(RuntimeError):
    """The reference's istat = -1 with its message."""


def _open(path):
    from scipy.io import netcdf_file

    return netcdf_file(path, "r", mmap=False)


def write_dbs(path, met, alt, lon=None, lat=None, topg=None, coord_sys="LON-LAT", title="synthetic"):
    """Writes a DBS.  ``met`` holds the fields on the DBS levels ``alt``:
    U V W T TP P QV RHO as (nt, nz, ny, nx), UST PBLH RMOL ZNT PRATE as
    (nt, ny, nx) (PRATE in mm/s), LDU as (ny, nx) and "times" (seconds after
    0000 UTC); names may also be given in lower case (u, v, w, t, tp, rho,
    ust, pblh, rmol, znt, prate, ldu, p, qv) as in the met series of
    ``synth``."""
    from scipy.io import netcdf_file

    def get(name):
        for k in (name, name.lower()):
            if k in met:
                return np.asarray(met[k])
        return None

    u = get("U")
    nt, nz, ny, nx = u.shape
    times = np.asarray(met["times"], dtype=np.float64)
    alt = np.asarray(alt, dtype=np.float32)
    assert alt.shape == (nz,) and times.shape == (nt,)
    f = netcdf_file(path, "w", version=2)  # NF90_64BIT_OFFSET
    xdim, ydim = ("lon", "lat") if coord_sys == "LON-LAT" else ("x", "y")
    f.createDimension(xdim, nx)
    f.createDimension(ydim, ny)
    f.createDimension("alt", nz)
    f.createDimension("time", nt)
    if lon is None:
        lon = np.arange(nx, dtype=np.float64)
    if lat is None:
        lat = np.arange(ny, dtype=np.float64)
    v = f.createVariable(xdim, "f4", (xdim,))
    v[:] = np.asarray(lon, dtype=np.float32)
    v = f.createVariable(ydim, "f4", (ydim,))
    v[:] = np.asarray(lat, dtype=np.float32)
    v = f.createVariable("alt", "f4", ("alt",))
    v[:] = alt
    v.units, v.description = b"m", b"height. Terrain following levels"
    v = f.createVariable("time", "f8", ("time",))
    v[:] = times
    v.units, v.description = b"s", b"time after 0000UTC"
    X, Y = np.meshgrid(np.asarray(lon, dtype=np.float32), np.asarray(lat, dtype=np.float32))
    static = {"XLON": X, "XLAT": Y, "UTM_X": X, "UTM_Y": Y,
              "TOPG": np.zeros((ny, nx)) if topg is None else np.asarray(topg),
              "LDU": get("LDU") if get("LDU") is not None else np.full((ny, nx), -99.0),
              "SOIL": np.zeros((ny, nx)), "VEGFRA": np.zeros((ny, nx))}
    for name in VARS_2D_STATIC:
        v = f.createVariable(name, "f4", (ydim, xdim))
        v[:] = np.asarray(static[name], dtype=np.float32)
    for name in VARS_2D_TIME:
        a = get(name)
        if a is None:
            continue
        v = f.createVariable(name, "f4", ("time", ydim, xdim))
        v[:] = np.asarray(a, dtype=np.float32)
    for name in VARS_3D:
        a = get(name)
        if a is None:
            continue
        v = f.createVariable(name, "f4", ("time", "alt", ydim, xdim))
        v[:] = np.asarray(a, dtype=np.float32)
    f.TITLE = f"Meteo database for Fall3d derived from {title}".encode()
    f.COORDINATES = coord_sys.encode()
    f.START_TIME = np.int32(int(times[0]))
    f.END_TIME = np.int32(int(times[-1]))
    f.TIME_INCREMENT = np.int32(int((times[-1] - times[0]) / (nt - 1)) if nt > 1 else 0)
    f.ZMIN = np.float32(alt[0])
    f.ZMAX = np.float32(alt[-1])
    f.NX, f.NY, f.NZ, f.NT = np.int32(nx), np.int32(ny), np.int32(nz), np.int32(nt)
    f.close()


def dbs_interval(times, timesec):
    """get_dbs_value_plane.f90:105-114: (itime, endsec), itime 0-based; the
    last interval [time(it), time(it+1)) that holds timesec, else the last
    record."""
    t = [int(x) for x in times]  # the reference reads the times into integers
    nt = len(t)
    if timesec < t[0] or timesec > t[nt - 1]:
        raise DBSError("get_dbs_value_plane: time not in the database interval")
    itime, endsec = nt - 1, t[nt - 1]
    for it in range(nt - 1):
        if t[it] <= timesec < t[it + 1]:
            itime, endsec = it, t[it + 1]
    return itime, endsec


def dbs_levels(alt, z):
    """get_dbs_value_plane.f90:140-155: (ialt1, ialt2, s), levels 0-based;
    the last pair of levels around z wins, z outside the levels takes the
    nearest one with s = 1."""
    alt = [float(a) for a in np.asarray(alt, dtype=np.float32)]
    nz = len(alt)
    if z <= alt[0]:
        return 0, 0, 1.0
    if z >= alt[nz - 1]:
        return nz - 1, nz - 1, 1.0
    ialt1 = ialt2 = None
    s = None
    for iz in range(nz - 1):
        if alt[iz] <= z <= alt[iz + 1]:
            ialt1, ialt2 = iz, iz + 1
            s = (z - alt[iz]) / (alt[iz + 1] - alt[iz])
    return ialt1, ialt2, s


def get_dbs_value_plane(ds, timesec, word, z):
    """libMaster/get_dbs_value_plane.f90: the (ny, nx) plane of ``word`` at
    time ``timesec`` and terrain-following height ``z`` (binary64), and the
    time until which it is valid.  ``ds`` is an open DBS (scipy netcdf_file)."""
    case = VARCASE.get(word)
    if case is None:
        raise DBSError(f"get_dbs_value_plane: word {word} not found in the dictionary")
    itime, endsec = dbs_interval(ds.variables["time"][:], timesec)
    if word not in ds.variables:
        raise DBSError(f"get_dbs_value_plane : Error getting netCDF ID for variable {word}")
    var = ds.variables[word]
    if case == 0:
        return np.asarray(var[:], dtype=np.float64), endsec
    if case == 1:
        return np.asarray(var[itime], dtype=np.float64), endsec
    i1, i2, s = dbs_levels(ds.variables["alt"][:], float(z))
    w1 = np.asarray(var[itime, i1], dtype=np.float64)
    w2 = np.asarray(var[itime, i2], dtype=np.float64)
    return (1.0 - s) * w1 + s * w2, endsec


def read_dbs(path, zlayer, wetdep=True, time_lag=0.0):
    """Sources/reamet.f90 for every record of the DBS: the met series of the
    context (f3d_met_series) on the model levels ``zlayer``.  Returns the
    dictionary (u, v, w, t, tp, rho, p, qv as (nt, nz, ny, nx); ust, pblh, rmol,
    znt, prate as (nt, ny, nx); ldu; times; time_lag) and the warnings the
    reference would have written."""
    ds = _open(path)
    try:
        times = np.asarray(ds.variables["time"][:], dtype=np.float64)
        nt = len(times)
        ny, nx = ds.variables["U"].shape[2:]
        zl = [float(z) for z in np.asarray(zlayer, dtype=np.float64)]
        nz = len(zl)
        out = {k: np.empty((nt, nz, ny, nx)) for k in ("u", "v", "w", "t", "tp", "p", "rho", "qv")}
        for k in ("ust", "pblh", "rmol", "znt", "prate"):
            out[k] = np.empty((nt, ny, nx))
        warnings = []
        names3 = {"u": "U", "v": "V", "w": "W", "t": "T", "tp": "TP", "p": "P", "rho": "RHO", "qv": "QV"}
        for it in range(nt):
            tsec = int(times[it])  # the record's own time: get_dbs_value_plane selects it
            for k, z in enumerate(zl):
                for key, word in names3.items():
                    if word not in ds.variables and key in ("qv", "p"):  # only aggregation reads them
                        out[key][it, k] = 0.0
                        continue
                    out[key][it, k], _ = get_dbs_value_plane(ds, tsec, word, z)
            out["ust"][it], _ = get_dbs_value_plane(ds, tsec, "UST", 0.0)
            out["rmol"][it], _ = get_dbs_value_plane(ds, tsec, "RMOL", 0.0)
            for key, word, default, what in (("pblh", "PBLH", 1500.0, "PBLH = 1.5km"),
                                             ("znt", "ZNT", 0.1, "ZNT = 0.1m")):
                try:
                    out[key][it], _ = get_dbs_value_plane(ds, tsec, word, 0.0)
                except DBSError:
                    out[key][it] = default
                    warnings.append(f"reamet : no value for {word}. Assuming {what}")
            if wetdep:
                try:
                    out["prate"][it], _ = get_dbs_value_plane(ds, tsec, "PRATE", 0.0)
                except DBSError:
                    out["prate"][it] = 0.0
                    warnings.append("reamet : no value for PRATE. Assuming PRATE = 0.0")
            else:
                out["prate"][it] = 0.0
        try:
            out["ldu"], _ = get_dbs_value_plane(ds, int(times[0]), "LDU", 0.0)
        except DBSError:
            out["ldu"] = np.full((ny, nx), -99.0)  # Master.f90:176
        out["times"] = times.astype(np.int32)
        out["time_lag"] = float(time_lag)
        return out, warnings
    finally:
        ds.close()


def _f90_max(a, b):
    """gfortran's MAX(a, b): b where b > a or a is a NaN."""
    return b if (b > a or math.isnan(a)) else a


def get_par_abl(z0, z1, tz0, tz1, pz0, pz1, u, v):
    """Utilities/SetDbs/get_par_ABL.f90: the friction velocity and the
    Monin-Obukhov length from two levels z0 < z1 (temperatures in K,
    pressures in Pa, the wind at z1) by the bulk Richardson number, in the
    reference's operation order (its exponent 0.285 is a binary32 literal,
    and the unstable branch's Gh uses the Gm updated just before it).
    Returns (ustar, rmonin)."""
    g, k = 9.81, 0.4
    e = float(np.float32(0.285))
    thz0 = tz0 * math.pow(1.01e5 / pz0, e)  # :34-35
    thz1 = tz1 * math.pow(1.01e5 / pz1, e)
    umod = _f90_max(math.sqrt(u * u + v * v), 1e-4)  # :39
    ri = ((g * (z1 - z0)) * (thz1 - thz0)) / (((umod * umod) * 0.5) * (tz0 + tz1))  # :43
    if ri >= 0.0:  # stable (:47-51)
        gm = 1.0 + 4.7 * ri
        gm = 1.0 / (gm * gm)
        gh = gm
    else:  # unstable (:53-59)
        gm = math.log(z1 / z0)
        gm = 1.0 + (((70.0 * k) * k) * math.sqrt((abs(ri) * z1) / z0)) / (gm * gm)
        gh = 1.0 + (((50.0 * k) * k) * math.sqrt((abs(ri) * z1) / z0)) / (gm * gm)
        gm = 1.0 - (9.4 * ri) / gm
        gh = 1.0 - (9.4 * ri) / gh
    ustar = math.log(z1 / z0)  # :63-64
    ustar = ((k * umod) * math.sqrt(gm)) / ustar
    thstar = math.log(z1 / z0)  # :68-70
    thstar = ((((k * k) * umod) * (thz1 - thz0)) * gh) / ((ustar * thstar) * thstar)
    thstar = _f90_max(thstar, 1e-4)
    rmonin = (((ustar * ustar) * 0.5) * (thz0 + thz1)) / ((k * g) * thstar)  # :74
    return ustar, rmonin


def debug_dbs(nx, ny, zlayer, times):
    """The met series of SetDbs's DEBUG model (read_DEBUG_data.f90 with its
    default, non-standard atmosphere and no wind rotation) for a DBS on the
    levels zlayer at the times (s): topography 0, u = 10 m/s, v = w = 0,
    T = Tv = Tp = 273 K, p = 1e5 Pa, rho = 1, qv = 0, PBLH = 1000 m, LDU =
    -999, ust and the Monin-Obukhov length L of each column from
    get_par_abl(1, zlayer(2), T(1), T(2), p(1), p(2), u(1), v(1)) (:97-102);
    RMOL, ZNT and PRATE keep SetDbs's initial 0 (Master.f90:178-179).
    Returns a dict for write_dbs (binary64 values; the file stores them in
    binary32)."""
    nt, nz = len(times), len(zlayer)
    shape3, shape2 = (nt, nz, ny, nx), (nt, ny, nx)
    T = np.full(shape3, 273.0)
    P = np.full(shape3, 1e5)
    # every column holds the same values, so one evaluation serves them all
    ust, lmo = get_par_abl(1.0, float(zlayer[1]), 273.0, 273.0, 1e5, 1e5, 10.0, 0.0)
    return {"U": np.full(shape3, 10.0), "V": np.zeros(shape3), "W": np.zeros(shape3), "T": T, "TP": T.copy(),
            "P": P, "QV": np.zeros(shape3), "RHO": np.ones(shape3), "PBLH": np.full(shape2, 1000.0),
            "UST": np.full(shape2, ust), "L": np.full(shape2, lmo), "RMOL": np.zeros(shape2),
            "ZNT": np.zeros(shape2), "PRATE": np.zeros(shape2), "LDU": np.full((ny, nx), -999.0),
            "times": np.asarray(times, dtype=np.float64)}
