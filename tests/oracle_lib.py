"""ctypes binding of the CPU oracle (oracle/f3d_oracle.cpp) for the tests,
smoke() and bench.py's CPU baseline.  The oracle checks the library's
results; the library never calls it."""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from fall3d_gb300 import _abi  # noqa: E402

D = C.c_double
I = C.c_int
DP = _abi.c_double_p
IP = _abi.c_int_p
VP = C.c_void_p

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_oracle  # noqa: E402

    path = build_oracle.build()
    lib = C.CDLL(path)
    sig = {
        "orc_setbcc": [DP, I, I, I, I, I, DP, DP, DP, DP, DP, DP, DP],
        "orc_advctzc": [DP, I, I, I, I, I, DP, DP, DP, D],
        "orc_advctx": [DP, I, I, I, I, I, DP, D, D],
        "orc_advcty": [DP, I, I, I, I, I, DP, D, D],
        "orc_diffz": [DP, I, I, I, I, I, DP, D, DP, DP],
        "orc_diffx": [DP, I, I, I, I, I, D, D, DP, DP],
        "orc_diffy": [DP, I, I, I, I, I, D, D, DP, DP],
        "orc_wetdep": [DP, DP, I, I, I, I, I, I, D, DP, DP, DP, DP, DP],
        "orc_accum": [DP, DP, I, I, I, I, I, I, D, DP, DP],
        "orc_clip": [DP, I, I, I, I, I],
        "orc_cmass2d": [DP, DP, DP, DP, DP, I, I, I, I, I, I, I, I, D, D, DP, D, DP],
        "orc_cmass3d": [DP, DP, DP, DP, I, I, I, I, D, D, DP, DP],
        "orc_getc0": [DP, DP, DP, I, I, I, I],
        "orc_setsrc": [DP, I, I, I, I, I, IP, IP, IP, DP, DP, DP, DP, D, D, D],
        "orc_finddt": [I, I, I, I, D, D, DP, DP, DP, DP, DP, DP, DP, DP, D, DP, DP],
        "orc_kappa3": [I, I, I, I, I, I, D, D, D, D, D, D, D, DP, DP, DP, DP, DP, DP, DP, DP, DP, DP,
                       DP],
        "orc_get_gama": [D, D, DP],
        "orc_vsettl": [D, D, D, D, DP, I, D, D, DP],
        "orc_setvset": [I, I, I, I, I, I, DP, DP, DP, DP, DP, DP, I, D, DP, DP, IP],
        "orc_setvdrydep": [I, I, I, DP, DP, DP, DP, DP, DP, DP, DP, DP],
        "orc_meteo_scale": [I, I, I, I, D, D, DP, DP, DP, DP, DP, DP, DP, DP, DP, DP],
        "orc_outputs": [DP, DP, I, I, I, I, DP, DP, DP, DP, DP],
        "orc_out_column": [DP, I, I, I, IP, I, DP, DP, DP],
        "orc_out_ground": [DP, I, I, I, IP, I, DP, DP],
        "orc_pm_classes": [I, DP, I, IP],
        "orc_out_aot": [DP, I, I, I, I, DP, DP, DP, DP, DP],
        "orc_out_thick": [DP, I, I, I, DP, DP, DP],
        "orc_standard_pressure": [D],
        "orc_setcut_fl": [I, I, I, DP, DP, DP, D],
        "orc_ter2asl": [DP, DP, DP, I, I, I],
        "orc_out_fl": [DP, I, I, I, I, DP, D, DP, DP],
        "orc_out_con": [DP, I, I, I, I, I, DP, DP, DP, I, DP],
        "orc_ctx_create": [VP, I],
        "orc_ctx_destroy": [VP],
        "orc_ctx_set_threads": [VP, I],
        "orc_meteo": [VP] + [DP] * 12,
        "orc_source": [VP, I, IP, IP, IP, DP],
        "orc_step": [VP],
        "orc_budget": [VP, DP],
        "orc_get_state": [VP, IP, DP],
        "orc_set_time": [VP, D, I],
        "orc_download": [VP, DP, DP, DP, DP, DP],
        "orc_upload_state": [VP, DP, DP, DP, D, D, D],
        "orc_download_coeffs": [VP] + [DP] * 7,
        "orc_download_iters": [VP, IP],
        "orc_outputs_ctx": [VP, DP, DP, DP],
        "orc_run_reset": [VP],
        "orc_set_gravity_current": [VP, VP],
        "orc_set_aggregation": [VP, D, I, DP],
        "orc_aggregation_met": [VP, DP, DP],
        "orc_aggregation_plume": [VP, I, IP, IP, IP, DP, DP],
        "orc_download_maggr": [VP, DP],
        "orc_track_points": [DP, DP, I, I, I, I, DP, DP, DP, DP, D, D, D, D, I, DP, DP, DP],
        "orc_run": [VP, VP, VP, D, D, I, VP, I, IP],
    }
    ret = {"orc_get_gama": I, "orc_vsettl": I, "orc_setvset": I, "orc_setsrc": I,
           "orc_ctx_create": VP, "orc_meteo": I, "orc_source": I, "orc_step": I, "orc_run": I,
           "orc_pm_classes": I, "orc_standard_pressure": D, "orc_set_aggregation": I, "orc_track_points": I}
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = ret.get(name, None)
    _lib = lib
    return lib


def p(a):
    return _abi.dptr(a)


def ip(a):
    return _abi.iptr(a)


def output(grid, fields, var, index=0, asl=False, p_levels=None, flight_level=None):
    """The oracle's printres_nc.f90 variable `var` (fall3d_gb300.OUT_*) of a
    state: fields = dict(c (nc, nz+2, ny+2, nx+2), cdry, cwet (nc+1, ny, nx))
    as f3d_download returns them; p_levels and flight_level for the cut."""
    import fall3d_gb300 as F

    lib = load()
    nx, ny, nz, nc, np_ = grid["nx"], grid["ny"], grid["nz"], grid["nc"], grid["np"]
    c = np.ascontiguousarray(fields["c"], dtype=np.float64)
    dz = np.ascontiguousarray(grid["dz"], dtype=np.float64)
    hm = np.ascontiguousarray(grid["Hm1"], dtype=np.float64)
    diam = np.ascontiguousarray(grid["diam"], dtype=np.float64)
    rhop = np.ascontiguousarray(grid["rhop"], dtype=np.float64)
    out2 = np.zeros((ny, nx))
    if var in (F.OUT_LOAD, F.OUT_WET, F.OUT_THICK):
        cdry = np.array(fields["cdry"], dtype=np.float64)
        cwet = np.array(fields["cwet"], dtype=np.float64)
        cload = np.zeros_like(cdry)
        lib.orc_getc0(p(cdry), p(cwet), p(cload), nx, ny, nc, np_)
        if var == F.OUT_THICK:
            lib.orc_out_thick(p(cload), nx, ny, np_, p(rhop), p(hm), p(out2))
            return out2
        f = cload if var == F.OUT_LOAD else cwet
        return f[index] / hm
    if var in (F.OUT_COL_MASS, F.OUT_C_GRND, F.OUT_PM_COL, F.OUT_PM_GRND):
        if var in (F.OUT_PM_COL, F.OUT_PM_GRND):
            cls = np.zeros(max(np_, 1), np.int32)
            n = lib.orc_pm_classes(np_, p(diam), int(index), ip(cls))
        elif var == F.OUT_COL_MASS and index > 0:
            cls, n = np.array([np_ + index - 1], np.int32), 1
        else:
            cls, n = np.arange(max(np_, 1), dtype=np.int32), np_
        if var in (F.OUT_COL_MASS, F.OUT_PM_COL):
            lib.orc_out_column(p(c), nx, ny, nz, ip(cls), n, p(dz), p(hm), p(out2))
        else:
            lib.orc_out_ground(p(c), nx, ny, nz, ip(cls), n, p(hm), p(out2))
        return out2
    if var == F.OUT_AOT05:
        lib.orc_out_aot(p(c), nx, ny, nz, np_, p(diam), p(rhop), p(dz), p(hm), p(out2))
        return out2
    if var == F.OUT_CON:
        out3 = np.zeros((nz, ny, nx))
        zl = np.ascontiguousarray(grid["zlayer"], dtype=np.float64)
        tg = np.ascontiguousarray(grid["topg"], dtype=np.float64)
        lib.orc_out_con(p(c), nx, ny, nz, np_, int(index), p(hm), p(zl), p(tg), int(bool(asl)), p(out3))
        return out3
    if var == "fl":
        pl = np.ascontiguousarray(p_levels, dtype=np.float64)
        lib.orc_out_fl(p(c), nx, ny, nz, np_, p(pl), float(flight_level), p(hm), p(out2))
        return out2
    raise ValueError(var)


def track_points(grid, fields, xpts, ypts, xo, yo):
    """The oracle's tracking-point values (orc_track_points) of a state as
    f3d_download returns it: (npts, 7 + 3*nz + 1 + np)."""
    lib = load()
    nx, ny, nz, nc, np_ = grid["nx"], grid["ny"], grid["nz"], grid["nc"], grid["np"]
    cdry = np.array(fields["cdry"], dtype=np.float64)
    cwet = np.array(fields["cwet"], dtype=np.float64)
    cload = np.zeros_like(cdry)
    lib.orc_getc0(p(cdry), p(cwet), p(cload), nx, ny, nc, np_)
    xp = np.ascontiguousarray(xpts, dtype=np.float64)
    yp = np.ascontiguousarray(ypts, dtype=np.float64)
    out = np.zeros((len(xp), 7 + 3 * nz + 1 + np_))
    rc = lib.orc_track_points(p(np.ascontiguousarray(fields["c"], dtype=np.float64)), p(cload), nx, ny, nz, np_,
                              p(np.ascontiguousarray(grid["diam"], dtype=np.float64)),
                              p(np.ascontiguousarray(grid["rhop"], dtype=np.float64)),
                              p(np.ascontiguousarray(grid["dz"], dtype=np.float64)),
                              p(np.ascontiguousarray(grid["Hm1"], dtype=np.float64)),
                              float(grid["dx"]), float(grid["dy"]), float(xo), float(yo), len(xp), p(xp), p(yp),
                              p(out))
    assert rc == 0, rc
    return out


class OracleCtx:
    """CPU mirror of the coarse context API (f3d_ctx_*)."""

    def __init__(self, scen, nthreads=1):
        self.lib = load()
        self.s = scen
        g = scen.grid
        self.nx, self.ny, self.nz, self.nc = g["nx"], g["ny"], g["nz"], g["nc"]
        self._grid = _abi.make_grid(g, 64)
        self.h = self.lib.orc_ctx_create(C.cast(C.pointer(self._grid.struct), VP), nthreads)

    def close(self):
        if self.h:
            self.lib.orc_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_threads(self, nthreads):
        """Threads of the class loop of the following steps."""
        self.lib.orc_ctx_set_threads(self.h, int(nthreads))

    def set_gravity_current(self, params=None):
        if params is None:
            self.lib.orc_set_gravity_current(self.h, None)
        else:
            self._gc = _abi.make_gravity_current(params)
            self.lib.orc_set_gravity_current(self.h, C.addressof(self._gc))

    def meteo(self, it=0):
        m = self.s.met
        f3 = [np.ascontiguousarray(m[k][it]) for k in ("u", "v", "w", "t", "tp", "rho")]
        f2 = [np.ascontiguousarray(m[k][it]) for k in ("ust", "pblh", "rmol", "znt", "prate")]
        rc = self.lib.orc_meteo(self.h, *[p(a) for a in f3 + f2], p(np.ascontiguousarray(m["ldu"])))
        assert rc == 0, rc

    def source(self, iint=0):
        sr = self.s.src
        off = int(np.sum(sr["nsou"][:iint]))
        n = int(sr["nsou"][iint])
        roff = off * self.nc
        isrc = np.ascontiguousarray(sr["isrc"][off:off + n])
        jsrc = np.ascontiguousarray(sr["jsrc"][off:off + n])
        ksrc = np.ascontiguousarray(sr["ksrc"][off:off + n])
        tm = np.ascontiguousarray(sr["tmrat"][roff:roff + n * self.nc])
        rc = self.lib.orc_source(self.h, n, ip(isrc), ip(jsrc), ip(ksrc), p(tm))
        assert rc == 0, rc

    def step(self):
        rc = self.lib.orc_step(self.h)
        assert rc == 0, rc

    def state(self):
        it = C.c_int()
        s = np.zeros(7)
        self.lib.orc_get_state(self.h, C.byref(it), p(s))
        return dict(iiter=it.value, time=s[0], dt=s[1], dtc=s[2], erumass=s[3], outmass=s[4],
                    flowrate=s[5], cd=s[6])

    def set_time(self, time, iiter):
        self.lib.orc_set_time(self.h, float(time), int(iiter))

    def fields(self):
        nx, ny, nz, nc = self.nx, self.ny, self.nz, self.nc
        c = np.zeros((nc, nz + 2, ny + 2, nx + 2))
        cdry = np.zeros((nc + 1, ny, nx))
        cwet = np.zeros((nc + 1, ny, nx))
        vset = np.zeros((nc, nz, ny, nx))
        vdep = np.zeros((nc, ny, nx))
        self.lib.orc_download(self.h, p(c), p(cdry), p(cwet), p(vset), p(vdep))
        return dict(c=c, cdry=cdry, cwet=cwet, vset=vset, vdep=vdep)

    def coeffs(self):
        s3 = (self.nz, self.ny, self.nx)
        arrs = [np.zeros(s3) for _ in range(7)]
        self.lib.orc_download_coeffs(self.h, *[p(a) for a in arrs])
        return dict(zip(("vx", "vy", "vz", "rho", "rkhor", "rkh1", "rkver"), arrs))

    def iters(self):
        it = np.zeros((self.nc, self.nz, self.ny, self.nx), np.int32)
        self.lib.orc_download_iters(self.h, ip(it))
        return it

    def budget(self):
        b = np.zeros(4)
        self.lib.orc_budget(self.h, p(b))
        return dict(massvol=b[0], massdep=b[1], massdry=b[2], masswet=b[3])

    def outputs(self):
        a = [np.zeros((self.ny, self.nx)) for _ in range(3)]
        self.lib.orc_outputs_ctx(self.h, *[p(x) for x in a])
        return dict(load=a[0], col_mass=a[1], c_grnd=a[2])

    def upload_state(self, c=None, cdry=None, cwet=None, erumass=0.0, outmass=0.0, cd=1.0):
        self.lib.orc_upload_state(self.h, p(c), p(cdry), p(cwet), erumass, outmass, cd)

    def set_aggregation(self, agg=None):
        """Aggregation in transport with synth.aggregation_inputs (None: off)."""
        self._agg = agg
        if agg is None:
            self.lib.orc_set_aggregation(self.h, 3.0, 1, None)
            return
        self._fc = np.ascontiguousarray(agg["fc"], dtype=np.float64)
        assert self.lib.orc_set_aggregation(self.h, float(agg["Df"]), int(agg["ndtagr"]), p(self._fc)) == 0

    def maggr(self):
        m = np.zeros((self.nz, self.ny, self.nx))
        self.lib.orc_download_maggr(self.h, p(m))
        return m

    def run(self, beg_time=None, end_time=None, max_steps=0, log_cap=4096):
        agg = getattr(self, "_agg", None)
        met = _abi.make_met(self.s.met, agg)
        src = _abi.make_src(self.s.src, agg)
        recs = (_abi.F3DLogRecord * log_cap)()
        n = C.c_int()
        rc = self.lib.orc_run(self.h, C.cast(met.ref(), VP), C.cast(src.ref(), VP),
                              self.s.beg_time if beg_time is None else beg_time,
                              self.s.end_time if end_time is None else end_time, int(max_steps),
                              C.cast(recs, VP), log_cap, C.byref(n))
        assert rc == 0, rc
        return _abi.log_array(recs, n.value)
