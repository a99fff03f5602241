"""fall3d_gb300 -- GB300-native transport step of FALL3D 7.0.

The compute path is the CUDA library ``libfall3d_gb300.so`` built in-tree for
sm_103a (``fall3d_gb300/build.py``); this module is its Python host mirror.
It exposes

* the fine-grained entry points with the reference subroutines' names and
  arguments (``setbcc``, ``advctzc``, ``advctx``, ... ``finddt``), which take
  numpy arrays (host memory, staged by the library) or CUDA tensors (device
  memory, used in place);
* ``Context``: one scenario resident on the GPU (``f3d_ctx_*``), driven by
  ``meteo``/``source``/``step`` or by the Fall3d.f90 time loop ``run``.

There is no CPU fallback: every call goes through the CUDA library, and
``load()`` raises if the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfall3d_gb300.so")

PREC_FP64, PREC_FP32 = 64, 32
OPT_FUSED, OPT_TILE, OPT_GRAPH, OPT_PREFETCH = 1, 2, 3, 4
# output variables of printres_nc.f90 (f3d_output)
(OUT_LOAD, OUT_WET, OUT_THICK, OUT_COL_MASS, OUT_PM_COL, OUT_C_GRND, OUT_PM_GRND, OUT_AOT05,
 OUT_CON, OUT_WIND, OUT_MAGGR) = range(1, 12)


class F3DError(RuntimeError):
    """A non-zero status returned by the CUDA library."""

    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None
I = C.c_int
D = C.c_double
VP = C.c_void_p
IP = C.POINTER(C.c_int)
DP = C.POINTER(C.c_double)


def load(build_if_missing: bool = False):
    """Loads the CUDA library (raising if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build as _b

            _b.build()
        else:
            raise ImportError(f"{LIB_PATH} is not built; run fall3d_gb300/build.py "
                              "(there is no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    fine = {
        "f3d_setbcc": [VP, IP, IP, IP, IP, IP, VP, VP, VP, VP, VP, VP, VP],
        "f3d_advctzc": [VP, IP, IP, IP, IP, IP, VP, VP, VP, DP, IP],
        "f3d_advctx": [VP, IP, IP, IP, IP, IP, VP, DP, DP, VP, IP],
        "f3d_advcty": [VP, IP, IP, IP, IP, IP, VP, DP, DP, VP, IP],
        "f3d_diffz": [VP, IP, IP, IP, IP, IP, VP, DP, VP, VP, VP],
        "f3d_diffx": [VP, IP, IP, IP, IP, IP, DP, DP, VP, VP, VP],
        "f3d_diffy": [VP, IP, IP, IP, IP, IP, DP, DP, VP, VP, VP],
        "f3d_wetdep": [VP, VP, IP, IP, IP, IP, IP, IP, DP, VP, VP, VP, VP, VP],
        "f3d_accum": [VP, VP, IP, IP, IP, IP, IP, IP, VP, DP, VP, VP],
        "f3d_clip": [VP, IP, IP, IP, IP, IP, IP],
        "f3d_cmass2d": [VP, VP, VP, VP, VP, IP, IP, IP, IP, IP, IP, IP, IP, DP, DP, VP, DP, DP],
        "f3d_cmass3d": [VP, VP, VP, VP, IP, IP, IP, IP, DP, DP, VP, DP, DP, DP, DP],
        "f3d_getc0": [VP, VP, VP, IP, IP, IP, IP],
        "f3d_setsrc": [VP, IP, IP, IP, IP, IP, VP, VP, VP, VP, VP, VP, VP, DP, DP, DP],
        "f3d_finddt": [IP, IP, IP, IP, DP, DP, VP, VP, VP, VP, VP, VP, VP, VP, DP, DP, DP],
        "f3d_kappa3": [IP, IP, IP, IP, IP, IP, DP, DP, DP, DP, DP, DP, DP, VP, VP, VP, VP, VP, VP,
                       VP, VP, VP, VP, VP],
        "f3d_setvset": [IP, IP, IP, IP, IP, IP, VP, VP, VP, VP, VP, VP, IP, DP, VP, DP],
        "f3d_setvdrydep": [IP, IP, IP, VP, VP, VP, VP, VP, VP, VP, VP, VP],
        "f3d_dmath_eval": [I, C.c_longlong, VP, VP],
        "f3d_meteo_scale": [IP, IP, IP, IP, DP, DP, VP, VP, VP, VP, VP, VP, VP, VP, VP, VP],
        "f3d_ctx_create": [VP, C.POINTER(VP)],
        "f3d_ctx_destroy": [VP],
        "f3d_ctx_footprint": [VP, C.POINTER(C.c_longlong)],
        "f3d_meteo": [VP] + [VP] * 12,
        "f3d_source": [VP, I, VP, VP, VP, VP],
        "f3d_step": [VP],
        "f3d_budget": [VP, DP, DP, DP, DP],
        "f3d_count_nonfinite": [VP, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)],
        "f3d_get_state": [VP, IP, DP, DP, DP, DP, DP, DP],
        "f3d_set_time": [VP, D, I],
        "f3d_download": [VP, VP, VP, VP, VP, VP],
        "f3d_upload_state": [VP, VP, VP, VP, D, D, D],
        "f3d_download_coeffs": [VP] + [VP] * 7,
        "f3d_download_iters": [VP, VP],
        "f3d_get_cd": [VP, DP],
        "f3d_outputs": [VP, VP, VP, VP],
        "f3d_output": [VP, I, I, I, VP, I],
        "f3d_output_fl": [VP, D, VP, VP, I],
        "f3d_set_gravity_current": [VP, VP],
        "f3d_set_aggregation": [VP, VP],
        "f3d_track_points": [VP, I, VP, VP, D, D, VP],
        "f3d_aggregation_met": [VP, VP, VP],
        "f3d_aggregation_plume": [VP, I, VP, VP, VP, VP, VP],
        "f3d_download_maggr": [VP, VP],
        "f3d_run": [VP, VP, VP, D, D, I, VP, I, IP],
        "f3d_run_reset": [VP],
        "f3d_sync": [VP],
        "f3d_last_error": [C.c_char_p, I],
        "f3d_ctx_stream": [VP, C.POINTER(VP)],
        "f3d_set_option": [VP, I, I],
        "f3d_get_option": [VP, I, IP],
        "f3d_profile_enable": [VP, I],
        "f3d_profile_read": [VP, I, C.c_char_p, I, C.POINTER(C.c_longlong), DP, IP],
        "f3d_ctx_save": [VP, C.c_char_p],
        "f3d_ctx_restore": [VP, C.c_char_p],
        "f3d_batch_create": [I, C.POINTER(VP)],
        "f3d_batch_destroy": [VP],
        "f3d_batch_add": [VP, VP, VP, VP, D, D, I, VP, I, IP],
        "f3d_batch_step": [VP, IP],
        "f3d_batch_poll": [VP, I, IP, IP, IP],
        "f3d_batch_release": [VP, I],
        "f3d_batch_sync": [VP],
        "f3d_batch_set_option": [VP, I, I],
        "f3d_batch_get_option": [VP, I, IP],
        "f3d_batch_autotune": [VP, I, IP, C.POINTER(C.c_float)],
        "f3d_batch_stats": [VP, C.POINTER(C.c_longlong), DP, IP],
        "f3d_batch_stream": [VP, C.POINTER(VP)],
        "f3d_cmass2d_noalloc": [VP, VP, VP, VP, VP, IP, IP, IP, IP, IP, IP, IP, IP, DP, DP, VP, DP, DP],
        "f3d_server_create": [C.c_longlong, I, C.POINTER(VP)],
        "f3d_server_destroy": [VP],
        "f3d_server_submit": [VP, VP, VP, VP, D, D, I, IP],
        "f3d_server_progress": [VP, I, IP, IP],
        "f3d_server_poll": [VP, I, IP, DP, DP, DP, C.POINTER(C.c_longlong)],
        "f3d_server_result": [VP, I, VP, VP, VP, VP, I, IP],
        "f3d_server_forget": [VP, I],
        "f3d_server_stats": [VP, C.POINTER(C.c_longlong), DP, C.POINTER(C.c_longlong), IP, IP],
        "f3d_server_batch": [VP, C.POINTER(VP)],
    }
    for name, args in fine.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = I
    lib.f3d_version.restype = C.c_char_p
    lib.f3d_version.argtypes = []
    lib.f3d_kernel_launches.restype = C.c_longlong
    lib.f3d_kernel_launches.argtypes = []
    _lib = lib
    return lib


def last_error() -> str:
    lib = load()
    buf = C.create_string_buffer(1024)
    lib.f3d_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def _check(rc):
    if rc != 0:
        raise F3DError(rc, last_error())


def kernel_launches() -> int:
    return int(load().f3d_kernel_launches())


def _addr(a):
    """Address of a numpy array (host) or a CUDA tensor (device); None -> NULL."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags.c_contiguous, "arrays must be C-contiguous"
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        assert a.is_contiguous(), "tensors must be contiguous"
        return a.data_ptr()
    raise TypeError(f"unsupported array type {type(a)}")


def _i(v):
    return C.byref(C.c_int(int(v)))


def _d(v):
    return C.byref(C.c_double(float(v)))


# ---------------------------------------------------------------------------
# Fine-grained entry points (reference subroutine argument lists).
# ---------------------------------------------------------------------------

def setbcc(c, nx, ny, nz, nz_loc, iz_loc, vx, vy, vz, vset, vdep, rkver, dz):
    """Sources/setbcc.f90:1 -- ghost layers of one class, in place."""
    _check(load().f3d_setbcc(_addr(c), _i(nx), _i(ny), _i(nz), _i(nz_loc), _i(iz_loc), _addr(vx),
                             _addr(vy), _addr(vz), _addr(vset), _addr(vdep), _addr(rkver), _addr(dz)))


def advctzc(c, nx, ny, nz, nz_loc, iz_loc, vz, vset, dz, dt, lmeth=1):
    """Sources/advctzc.f90:1 -- vertical advection + settling, in place."""
    _check(load().f3d_advctzc(_addr(c), _i(nx), _i(ny), _i(nz), _i(nz_loc), _i(iz_loc), _addr(vz),
                              _addr(vset), _addr(dz), _d(dt), _i(lmeth)))


def advctx(c, nx, ny, nz, nz_loc, iz_loc, vx, dx, dt, work=None, lmeth=1):
    """Sources/advctx.f90:1"""
    _check(load().f3d_advctx(_addr(c), _i(nx), _i(ny), _i(nz), _i(nz_loc), _i(iz_loc), _addr(vx),
                             _d(dx), _d(dt), None, _i(lmeth)))


def advcty(c, nx, ny, nz, nz_loc, iz_loc, vy, dy, dt, work=None, lmeth=1):
    """Sources/advcty.f90:1"""
    _check(load().f3d_advcty(_addr(c), _i(nx), _i(ny), _i(nz), _i(nz_loc), _i(iz_loc), _addr(vy),
                             _d(dy), _d(dt), None, _i(lmeth)))


def diffz(c, nx, ny, nz, nz_loc, iz_loc, dz, dt, rkver, rho, work=None):
    """Sources/diffz.f90:1"""
    _check(load().f3d_diffz(_addr(c), _i(nx), _i(ny), _i(nz), _i(nz_loc), _i(iz_loc), _addr(dz),
                            _d(dt), _addr(rkver), _addr(rho), None))


def diffx(c, nx, ny, nz, nz_loc, iz_loc, dx, dt, rkhor, rho, work=None):
    """Sources/diffx.f90:1"""
    _check(load().f3d_diffx(_addr(c), _i(nx), _i(ny), _i(nz), _i(nz_loc), _i(iz_loc), _d(dx), _d(dt),
                            _addr(rkhor), _addr(rho), None))


def diffy(c, nx, ny, nz, nz_loc, iz_loc, dy, dt, rkhor, rho, work=None):
    """Sources/diffy.f90:1"""
    _check(load().f3d_diffy(_addr(c), _i(nx), _i(ny), _i(nz), _i(nz_loc), _i(iz_loc), _d(dy), _d(dt),
                            _addr(rkhor), _addr(rho), None))


def wetdep(c, cwet, ic, nx, ny, nz, nz_loc, iz_loc, dt, diam, zlayer, dz, zi, prate):
    """Sources/wetdep.f90:1 (cwet is the whole (nx,ny,0:nc) array; ic 1-based)."""
    _check(load().f3d_wetdep(_addr(c), _addr(cwet), _i(ic), _i(nx), _i(ny), _i(nz), _i(nz_loc),
                             _i(iz_loc), _d(dt), _addr(diam), _addr(zlayer), _addr(dz), _addr(zi),
                             _addr(prate)))


def accum(c, cdry, ic, nx, ny, nz, nz_loc, iz_loc, vz, dt, vset, vdep):
    """Sources/accum.f90:1 (cdry is the whole (nx,ny,0:nc) array; ic 1-based)."""
    _check(load().f3d_accum(_addr(c), _addr(cdry), _i(ic), _i(nx), _i(ny), _i(nz), _i(nz_loc),
                            _i(iz_loc), _addr(vz), _d(dt), _addr(vset), _addr(vdep)))


def clip(c, nx, ny, nz, nc, ic_loc=1, nc_loc=None):
    """Sources/sizloop.f90:77-78"""
    _check(load().f3d_clip(_addr(c), _i(nx), _i(ny), _i(nz), _i(nc), _i(ic_loc),
                           _i(nc if nc_loc is None else nc_loc)))


def cmass2d(c, vx, vy, vz, vset, nx, ny, nz, nc, ic_loc, nc_loc, iz_loc, nz_loc, dx, dy, dz, dt,
            outmass):
    """Sources/cmass2d.f90:1 -- returns outmass + outflow of the step."""
    om = C.c_double(float(outmass))
    _check(load().f3d_cmass2d(_addr(c), _addr(vx), _addr(vy), _addr(vz), _addr(vset), _i(nx), _i(ny),
                              _i(nz), _i(nc), _i(ic_loc), _i(nc_loc), _i(iz_loc), _i(nz_loc), _d(dx),
                              _d(dy), _addr(dz), _d(dt), C.byref(om)))
    return om.value


def cmass3d(c, cload, cdry, cwet, nx, ny, nz, nc, dx, dy, dz):
    """Sources/cmass3d.f90:1 -- (massvol, massdep, massdry, masswet)."""
    out = [C.c_double() for _ in range(4)]
    _check(load().f3d_cmass3d(_addr(c), _addr(cload), _addr(cdry), _addr(cwet), _i(nx), _i(ny), _i(nz),
                              _i(nc), _d(dx), _d(dy), _addr(dz), *[C.byref(o) for o in out]))
    return tuple(o.value for o in out)


def getc0(cdry, cwet, cload, nx, ny, nc, np_):
    """Sources/endstep.f90:80 getc0 + cload = cdry + cwet."""
    _check(load().f3d_getc0(_addr(cdry), _addr(cwet), _addr(cload), _i(nx), _i(ny), _i(nc), _i(np_)))


def setsrc(c, nx, ny, nz, nc, nsou, isrc, jsrc, ksrc, tmrat, dz, zlayer, Hm1, dX1, dX2, dt):
    """Sources/setsrc.f90:1 (tmrat already scaled by Hm1)."""
    _check(load().f3d_setsrc(_addr(c), _i(nx), _i(ny), _i(nz), _i(nc), _i(nsou), _addr(isrc),
                             _addr(jsrc), _addr(ksrc), _addr(tmrat), _addr(dz), _addr(zlayer),
                             _addr(Hm1), _d(dX1), _d(dX2), _d(dt)))


def finddt(nx, ny, nz, nc, dX1, dX2, dz, vx, vy, vz, vset, rkh1, rkhor, rkver, safety_factor=0.9):
    """Sources/finddt.f90:1 -- returns (dt, dtc)."""
    dt, dtc = C.c_double(), C.c_double()
    _check(load().f3d_finddt(_i(nx), _i(ny), _i(nz), _i(nc), _d(dX1), _d(dX2), _addr(dz), _addr(vx),
                             _addr(vy), _addr(vz), _addr(vset), _addr(rkh1), _addr(rkhor), _addr(rkver),
                             _d(safety_factor), C.byref(dt), C.byref(dtc)))
    return dt.value, dtc.value


def kappa3(nx, ny, nz, modkv, modkh, coord_sys, rkv0, rkh0, Csh, dX1, dX2, dx, dy, dz, zlayer, Hm1,
           vx, vy, vptemp, ustar, zi, rl, rkver, rkhor):
    """Sources/kappa3.f90:1 (rkver, rkhor in/out)."""
    _check(load().f3d_kappa3(_i(nx), _i(ny), _i(nz), _i(modkv), _i(modkh), _i(coord_sys), _d(rkv0),
                             _d(rkh0), _d(Csh), _d(dX1), _d(dX2), _d(dx), _d(dy), _addr(dz),
                             _addr(zlayer), _addr(Hm1), _addr(vx), _addr(vy), _addr(vptemp),
                             _addr(ustar), _addr(zi), _addr(rl), _addr(rkver), _addr(rkhor)))


def setvset(nx, ny, nz, nc, np_, modv, diam, rhop, psi, sphe, tempe, rho, aggregate, vset_factor,
            vset, cd):
    """Sources/setvset.f90:1 with the SAVEd cd made explicit; returns the exit cd."""
    cdv = C.c_double(float(cd))
    _check(load().f3d_setvset(_i(nx), _i(ny), _i(nz), _i(nc), _i(np_), _i(modv), _addr(diam),
                              _addr(rhop), _addr(psi), _addr(sphe), _addr(tempe), _addr(rho),
                              _i(aggregate), _d(vset_factor), _addr(vset), C.byref(cdv)))
    return cdv.value


def dmath_eval(op, x):
    """Diagnostic: the drag iteration's table-driven binary64 log (op 0) or
    exp (op 1) of every value of the float64 array x, or (op 2) the
    quotients a/b of the pairs x = (a0, b0, a1, b1, ...) formed from the
    reciprocal of b as the plain form's sweeps divide.  Returns a new
    array (one value per pair for op 2)."""
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    if op == 2:
        if x.size % 2:
            raise ValueError("op 2 takes pairs: x must have an even number of values")
        n = x.size // 2
    else:
        n = x.size
    y = np.empty(n, dtype=np.float64)
    _check(load().f3d_dmath_eval(int(op), n, _addr(x), _addr(y)))
    return y


def setvdrydep(nx, ny, nc, diam, zlayer, ldu, rl, znt, ustar, tempe, rho, vdep):
    """Sources/setvdrydep.f90:1 (tempe, rho: the k=1 plane)."""
    _check(load().f3d_setvdrydep(_i(nx), _i(ny), _i(nc), _addr(diam), _addr(zlayer), _addr(ldu),
                                 _addr(rl), _addr(znt), _addr(ustar), _addr(tempe), _addr(rho),
                                 _addr(vdep)))


def meteo_scale(nx, ny, nz, coord_sys, dX1, dX2, dz, Hm1, topg, vx, vy, vz, rho, rkhor, rkh1, divu):
    """Sources/meteo.f90:108-123 + corvver.f90 + setdivu.f90 (in place)."""
    _check(load().f3d_meteo_scale(_i(nx), _i(ny), _i(nz), _i(coord_sys), _d(dX1), _d(dX2), _addr(dz),
                                  _addr(Hm1), _addr(topg), _addr(vx), _addr(vy), _addr(vz), _addr(rho),
                                  _addr(rkhor), _addr(rkh1), _addr(divu)))


# ---------------------------------------------------------------------------
# Coarse context.
# ---------------------------------------------------------------------------

class Context:
    """One scenario resident on the GPU (the coarse C API, f3d_ctx_*)."""

    def __init__(self, scen, precision: int = PREC_FP64):
        self.lib = load()
        self.s = scen
        g = scen.grid
        self.nx, self.ny, self.nz, self.nc = g["nx"], g["ny"], g["nz"], g["nc"]
        self.precision = precision
        self._grid = _abi.make_grid(g, precision)
        h = VP()
        _check(self.lib.f3d_ctx_create(C.addressof(self._grid.struct), C.byref(h)))
        self.h = h

    @staticmethod
    def footprint(scen, precision=PREC_FP64) -> int:
        g = _abi.make_grid(scen.grid, precision)
        b = C.c_longlong()
        _check(load().f3d_ctx_footprint(C.addressof(g.struct), C.byref(b)))
        return int(b.value)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.f3d_ctx_destroy(self.h)
            self.h = VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- meteorology / sources / step -----------------------------------
    def meteo(self, it=0, fields=None):
        """meteo.f90:19-149 for DBS snapshot ``it`` of the scenario (or for an
        explicit dict of raw fields, numpy or CUDA tensors)."""
        if fields is None:
            m = self.s.met
            fields = {k: np.ascontiguousarray(m[k][it]) for k in
                      ("u", "v", "w", "t", "tp", "rho", "ust", "pblh", "rmol", "znt", "prate")}
            fields["ldu"] = np.ascontiguousarray(m["ldu"])
        keys = ("u", "v", "w", "t", "tp", "rho", "ust", "pblh", "rmol", "znt", "prate", "ldu")
        _check(self.lib.f3d_meteo(self.h, *[_addr(fields.get(k)) for k in keys]))

    def source(self, iint=0):
        """source.f90 for interval ``iint`` of the scenario's source series."""
        sr = self.s.src
        off = int(np.sum(sr["nsou"][:iint]))
        n = int(sr["nsou"][iint])
        arrs = [np.ascontiguousarray(sr[k][off:off + n], dtype=np.int32) for k in ("isrc", "jsrc", "ksrc")]
        tm = np.ascontiguousarray(sr["tmrat"][off * self.nc:(off + n) * self.nc])
        _check(self.lib.f3d_source(self.h, n, *[_addr(a) for a in arrs], _addr(tm)))

    def step(self, n=1):
        for _ in range(n):
            _check(self.lib.f3d_step(self.h))

    def sync(self):
        _check(self.lib.f3d_sync(self.h))

    def set_time(self, time, iiter):
        _check(self.lib.f3d_set_time(self.h, float(time), int(iiter)))

    # -- state -------------------------------------------------------------
    def state(self):
        it = C.c_int()
        v = [C.c_double() for _ in range(6)]
        _check(self.lib.f3d_get_state(self.h, C.byref(it), *[C.byref(x) for x in v]))
        cd = C.c_double()
        _check(self.lib.f3d_get_cd(self.h, C.byref(cd)))
        t, dt, dtc, eru, out, fr = (x.value for x in v)
        return dict(iiter=it.value, time=t, dt=dt, dtc=dtc, erumass=eru, outmass=out, flowrate=fr,
                    cd=cd.value)

    def fields(self):
        nx, ny, nz, nc = self.nx, self.ny, self.nz, self.nc
        c = np.zeros((nc, nz + 2, ny + 2, nx + 2))
        cdry = np.zeros((nc + 1, ny, nx))
        cwet = np.zeros((nc + 1, ny, nx))
        vset = np.zeros((nc, nz, ny, nx))
        vdep = np.zeros((nc, ny, nx))
        _check(self.lib.f3d_download(self.h, _addr(c), _addr(cdry), _addr(cwet), _addr(vset),
                                     _addr(vdep)))
        return dict(c=c, cdry=cdry, cwet=cwet, vset=vset, vdep=vdep)

    def download_c(self, out):
        """Concentrations into ``out`` (numpy or CUDA float64, (nc,nz+2,ny+2,nx+2))."""
        _check(self.lib.f3d_download(self.h, _addr(out), None, None, None, None))

    def coeffs(self):
        arrs = [np.zeros((self.nz, self.ny, self.nx)) for _ in range(7)]
        _check(self.lib.f3d_download_coeffs(self.h, *[_addr(a) for a in arrs]))
        return dict(zip(("vx", "vy", "vz", "rho", "rkhor", "rkh1", "rkver"), arrs))

    def iters(self):
        it = np.zeros((self.nc, self.nz, self.ny, self.nx), np.int32)
        _check(self.lib.f3d_download_iters(self.h, _addr(it)))
        return it

    def budget(self):
        v = [C.c_double() for _ in range(4)]
        _check(self.lib.f3d_budget(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("massvol", "massdep", "massdry", "masswet"), (x.value for x in v)))

    def count_nonfinite(self):
        """(NaN or infinite values in c, in cdry + cwet) on the device."""
        a, b = C.c_longlong(), C.c_longlong()
        _check(self.lib.f3d_count_nonfinite(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def outputs(self):
        a = [np.zeros((self.ny, self.nx)) for _ in range(3)]
        _check(self.lib.f3d_outputs(self.h, *[_addr(x) for x in a]))
        return dict(load=a[0], col_mass=a[1], c_grnd=a[2])

    def set_gravity_current(self, params=None):
        """GRAVITY_CURRENT = YES with the parameters of synth.gravity_current
        (a dict with the f3d_gravity_current fields); None switches it off."""
        if params is None:
            _check(self.lib.f3d_set_gravity_current(self.h, None))
        else:
            st = _abi.make_gravity_current(params)
            _check(self.lib.f3d_set_gravity_current(self.h, C.addressof(st)))

    def set_aggregation(self, agg=None):
        """Aggregation in transport with the inputs of synth.aggregation_inputs
        (Df, ndtagr, fc; the QV/P snapshots and plume lists are passed by
        run()); None switches it off."""
        self._agg = agg
        if agg is None:
            _check(self.lib.f3d_set_aggregation(self.h, None))
            return
        self._agg_fc = np.ascontiguousarray(agg["fc"], dtype=np.float64)
        st = _abi.F3DAggregation(Df=float(agg["Df"]), ndtagr=int(agg["ndtagr"]),
                                 fc=_abi.dptr(self._agg_fc))
        _check(self.lib.f3d_set_aggregation(self.h, C.addressof(st)))

    def maggr(self):
        m = np.zeros((self.nz, self.ny, self.nx))
        _check(self.lib.f3d_download_maggr(self.h, m.ctypes.data))
        return m

    def output(self, var, index=0, asl=False, binary32=False):
        """One output variable of printres_nc.f90 (OUT_*): (ny, nx), or
        (nz, ny, nx) for OUT_CON; binary32 as the netCDF file holds it."""
        shape = (self.nz, self.ny, self.nx) if var in (OUT_CON, OUT_WIND, OUT_MAGGR) else (self.ny, self.nx)
        a = np.zeros(shape, np.float32 if binary32 else np.float64)
        _check(self.lib.f3d_output(self.h, int(var), int(index), int(bool(asl)), a.ctypes.data,
                                   1 if binary32 else 0))
        return a

    def track_points(self, xpts, ypts, xo, yo):
        """Tracking-point values (f3d_track_points) at points (x, y) of the
        grid's coordinates with origin (xo, yo): (npts, 7 + 3*nz + 1 + np)."""
        xp = np.ascontiguousarray(xpts, dtype=np.float64)
        yp = np.ascontiguousarray(ypts, dtype=np.float64)
        out = np.zeros((len(xp), 7 + 3 * self.nz + 1 + self.s.grid.get("np", self.nc)))
        _check(self.lib.f3d_track_points(self.h, len(xp), xp.ctypes.data, yp.ctypes.data, float(xo), float(yo),
                                         out.ctypes.data))
        return out

    def output_fl(self, flight_level, p, binary32=False):
        """Particle concentration at a flight level (hundreds of feet), with
        p the pressure (nz, ny, nx) of the model levels in Pa."""
        p = np.ascontiguousarray(p, dtype=np.float64)
        assert p.shape == (self.nz, self.ny, self.nx)
        a = np.zeros((self.ny, self.nx), np.float32 if binary32 else np.float64)
        _check(self.lib.f3d_output_fl(self.h, float(flight_level), p.ctypes.data, a.ctypes.data,
                                      1 if binary32 else 0))
        return a

    def upload_state(self, c=None, cdry=None, cwet=None, erumass=0.0, outmass=0.0, cd=1.0):
        _check(self.lib.f3d_upload_state(self.h, _addr(c), _addr(cdry), _addr(cwet), float(erumass),
                                         float(outmass), float(cd)))

    # -- the Fall3d.f90 time loop -------------------------------------------
    def run(self, beg_time=None, end_time=None, max_steps=0, log_cap=4096, met=None, src=None):
        """Sources/Fall3d.f90:73-121 on the device; returns the mass-budget log."""
        agg = getattr(self, "_agg", None)
        met = met or _abi.make_met(self.s.met, agg)
        src = src or _abi.make_src(self.s.src, agg)
        recs = (_abi.F3DLogRecord * log_cap)()
        n = C.c_int()
        _check(self.lib.f3d_run(self.h, C.addressof(met.struct), C.addressof(src.struct),
                                self.s.beg_time if beg_time is None else float(beg_time),
                                self.s.end_time if end_time is None else float(end_time),
                                int(max_steps), C.addressof(recs), log_cap, C.byref(n)))
        return _abi.log_array(recs, n.value)

    def save(self, path):
        """Lossless checkpoint of the run's state (f3d_ctx_save)."""
        _check(self.lib.f3d_ctx_save(self.h, str(path).encode()))

    def restore(self, path):
        """Restores a checkpoint; the next run() continues the saved run."""
        _check(self.lib.f3d_ctx_restore(self.h, str(path).encode()))

    def run_reset(self):
        _check(self.lib.f3d_run_reset(self.h))

    def set_option(self, key: int, value: int):
        _check(self.lib.f3d_set_option(self.h, int(key), int(value)))

    def get_option(self, key: int) -> int:
        v = C.c_int()
        _check(self.lib.f3d_get_option(self.h, int(key), C.byref(v)))
        return v.value

    # -- timing ------------------------------------------------------------
    def stream_handle(self) -> int:
        """The cudaStream_t of this context (for CUDA events on it)."""
        p = VP()
        _check(self.lib.f3d_ctx_stream(self.h, C.byref(p)))
        return int(p.value or 0)

    def profile(self, enable: bool = True):
        _check(self.lib.f3d_profile_enable(self.h, int(enable)))

    def profile_read(self):
        """{kernel: (launches, total_ms)} recorded with CUDA events on the
        context's stream since profile(True)."""
        cap, nl = 64, 32
        names = C.create_string_buffer(cap * nl)
        cnt = (C.c_longlong * cap)()
        ms = (C.c_double * cap)()
        nk = C.c_int()
        _check(self.lib.f3d_profile_read(self.h, cap, names, nl, cnt, ms, C.byref(nk)))
        out = {}
        for i in range(min(nk.value, cap)):
            nm = names.raw[i * nl:(i + 1) * nl].split(b"\0", 1)[0].decode()
            out[nm] = (int(cnt[i]), float(ms[i]))
        return out


def version() -> str:
    return load().f3d_version().decode()


class Batch:
    """The batched precision form (f3d_batch_*): the time loops of many
    precision-form contexts advanced together, one persistent launch (one
    CUDA graph replay) per batch step."""

    DONE, RUNNING, FAILED = 2, 1, 3

    def __init__(self, max_scenarios: int):
        self.lib = load()
        h = VP()
        _check(self.lib.f3d_batch_create(int(max_scenarios), C.byref(h)))
        self.h = h
        self._keep = {}  # slot -> (ctx, met, src, log records): alive while in the batch

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.f3d_batch_destroy(self.h)
            self.h = VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, ctx: "Context", beg_time=None, end_time=None, max_steps=0, log_cap=4096, met=None,
            src=None) -> int:
        met = met or _abi.make_met(ctx.s.met)
        src = src or _abi.make_src(ctx.s.src)
        recs = (_abi.F3DLogRecord * log_cap)()
        slot = C.c_int()
        _check(self.lib.f3d_batch_add(self.h, ctx.h, C.addressof(met.struct), C.addressof(src.struct),
                                      ctx.s.beg_time if beg_time is None else float(beg_time),
                                      ctx.s.end_time if end_time is None else float(end_time),
                                      int(max_steps), C.addressof(recs), int(log_cap), C.byref(slot)))
        self._keep[slot.value] = (ctx, met, src, recs)
        return slot.value

    def step(self) -> int:
        n = C.c_int()
        _check(self.lib.f3d_batch_step(self.h, C.byref(n)))
        return n.value

    def run(self) -> None:
        """Steps until no scenario is running."""
        while self.step() > 0:
            pass

    def poll(self, slot: int):
        """(state, steps, log records so far)."""
        st, steps, nlog = C.c_int(), C.c_int(), C.c_int()
        _check(self.lib.f3d_batch_poll(self.h, int(slot), C.byref(st), C.byref(steps), C.byref(nlog)))
        return st.value, steps.value, nlog.value

    def log(self, slot: int):
        _, _, nlog = self.poll(slot)
        return _abi.log_array(self._keep[slot][3], nlog)

    def release(self, slot: int):
        _check(self.lib.f3d_batch_release(self.h, int(slot)))
        self._keep.pop(slot, None)

    def sync(self):
        _check(self.lib.f3d_batch_sync(self.h))

    def set_option(self, key: int, value: int):
        _check(self.lib.f3d_batch_set_option(self.h, int(key), int(value)))

    def get_option(self, key: int) -> int:
        v = C.c_int()
        _check(self.lib.f3d_batch_get_option(self.h, int(key), C.byref(v)))
        return v.value

    def autotune(self, reps: int = 3):
        """Picks the fastest tile shape on the running scenarios; returns
        (best shape, [ms per shape])."""
        best = C.c_int()
        ms = (C.c_float * 4)()
        _check(self.lib.f3d_batch_autotune(self.h, int(reps), C.byref(best), ms))
        return best.value, [float(v) for v in ms]

    def stats(self):
        """(batch steps, cell-class-steps, running scenarios)."""
        bs, cc, n = C.c_longlong(), C.c_double(), C.c_int()
        _check(self.lib.f3d_batch_stats(self.h, C.byref(bs), C.byref(cc), C.byref(n)))
        return bs.value, cc.value, n.value

    def stream_handle(self) -> int:
        p = VP()
        _check(self.lib.f3d_batch_stream(self.h, C.byref(p)))
        return int(p.value or 0)


class Server:
    """The serving form (f3d_server_*): continuous batching of forecast
    requests under an HBM admission cap."""

    QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3

    def __init__(self, hbm_cap_bytes: int, max_running: int = 128):
        self.lib = load()
        h = VP()
        _check(self.lib.f3d_server_create(int(hbm_cap_bytes), int(max_running), C.byref(h)))
        self.h = h
        self._keep = {}

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.f3d_server_destroy(self.h)
            self.h = VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, scen, log_cap: int = 1024) -> int:
        grid = _abi.make_grid(scen.grid, PREC_FP32)
        met = _abi.make_met(scen.met)
        src = _abi.make_src(scen.src)
        rid = C.c_int()
        _check(self.lib.f3d_server_submit(self.h, C.addressof(grid.struct), C.addressof(met.struct),
                                          C.addressof(src.struct), float(scen.beg_time),
                                          float(scen.end_time), int(log_cap), C.byref(rid)))
        self._keep[rid.value] = (grid, met, src, scen.grid["nx"], scen.grid["ny"])
        return rid.value

    def progress(self, max_steps: int = 1):
        """(running, queued) after admitting and up to max_steps batch steps."""
        r, q = C.c_int(), C.c_int()
        _check(self.lib.f3d_server_progress(self.h, int(max_steps), C.byref(r), C.byref(q)))
        return r.value, q.value

    def poll(self, rid: int):
        """dict(state, t_submit, t_admit, t_done, steps); a failed request
        raises F3DError."""
        st, steps = C.c_int(), C.c_longlong()
        ts, ta, td = C.c_double(), C.c_double(), C.c_double()
        rc = self.lib.f3d_server_poll(self.h, int(rid), C.byref(st), C.byref(ts), C.byref(ta), C.byref(td),
                                      C.byref(steps))
        if rc and st.value != self.FAILED:
            _check(rc)
        return dict(state=st.value, t_submit=ts.value, t_admit=ta.value, t_done=td.value,
                    steps=steps.value, error=last_error() if rc else "")

    def result(self, rid: int, log_cap: int = 1024):
        """LOAD, COL_MASS, C_GRND (ny, nx) and the mass-budget log; frees the
        request's host arrays of the submission."""
        _, _, _, nx, ny = self._keep[rid]
        load, col, grnd = (np.zeros((ny, nx)) for _ in range(3))
        recs = (_abi.F3DLogRecord * log_cap)()
        n = C.c_int()
        _check(self.lib.f3d_server_result(self.h, int(rid), _addr(load), _addr(col), _addr(grnd),
                                          C.addressof(recs), int(log_cap), C.byref(n)))
        return dict(load=load, col_mass=col, c_grnd=grnd, log=_abi.log_array(recs, min(n.value, log_cap)))

    def forget(self, rid: int):
        _check(self.lib.f3d_server_forget(self.h, int(rid)))
        self._keep.pop(rid, None)

    def stats(self):
        used, bs = C.c_longlong(), C.c_longlong()
        ccs = C.c_double()
        r, q = C.c_int(), C.c_int()
        _check(self.lib.f3d_server_stats(self.h, C.byref(used), C.byref(ccs), C.byref(bs), C.byref(r),
                                         C.byref(q)))
        return dict(used_bytes=used.value, cell_class_steps=ccs.value, batch_steps=bs.value,
                    running=r.value, queued=q.value)
