"""ctypes mirrors of the structs in include/fall3d_gpu.h.

The C structs hold raw pointers; ``Pinned`` keeps the numpy arrays they point
into alive for as long as the struct is used.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)


class F3DGrid(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("nc", C.c_int), ("np", C.c_int),
        ("coord_sys", C.c_int), ("modkv", C.c_int), ("modkh", C.c_int), ("modv", C.c_int),
        ("wetdep", C.c_int), ("aggregate", C.c_int), ("precision", C.c_int),
        ("dX1", C.c_double), ("dX2", C.c_double), ("dx", C.c_double), ("dy", C.c_double),
        ("rkh0", C.c_double), ("rkv0", C.c_double), ("Csh", C.c_double),
        ("safety_factor", C.c_double), ("vset_factor", C.c_double),
        ("dz", c_double_p), ("zlayer", c_double_p), ("Hm1", c_double_p), ("topg", c_double_p),
        ("diam", c_double_p), ("rhop", c_double_p), ("psi", c_double_p), ("sphe", c_double_p),
    ]


class F3DMetSeries(C.Structure):
    _fields_ = [
        ("nt", C.c_int), ("times", c_int_p), ("time_lag", C.c_double),
        ("u", c_double_p), ("v", c_double_p), ("w", c_double_p), ("t", c_double_p),
        ("tp", c_double_p), ("rho", c_double_p),
        ("ust", c_double_p), ("pblh", c_double_p), ("rmol", c_double_p), ("znt", c_double_p),
        ("prate", c_double_p), ("ldu", c_double_p), ("qv", c_double_p), ("p", c_double_p),
    ]


class F3DSrcSeries(C.Structure):
    _fields_ = [
        ("nint", C.c_int), ("t1", c_int_p), ("t2", c_int_p), ("nsou", c_int_p),
        ("isrc", c_int_p), ("jsrc", c_int_p), ("ksrc", c_int_p), ("tmrat", c_double_p),
        ("nplume", c_int_p), ("pix", c_int_p), ("piy", c_int_p), ("piz", c_int_p),
        ("ptemp", c_double_p), ("pwater", c_double_p),
    ]


class F3DGravityCurrent(C.Structure):
    """f3d_gravity_current (include/fall3d_gpu.h)."""

    _fields_ = [(n, C.c_double) for n in ("c_flow_rate", "lambda_grav", "k_entrain", "brunt_vaisala",
                                          "center_x", "center_y", "xorigr", "yorigr", "h_tot",
                                          "beg_time")]


class F3DAggregation(C.Structure):
    """f3d_aggregation (include/fall3d_gpu.h)."""

    _fields_ = [("Df", C.c_double), ("ndtagr", C.c_int), ("fc", c_double_p)]


def make_gravity_current(p: dict) -> F3DGravityCurrent:
    return F3DGravityCurrent(**{k: float(p[k]) for k, _ in F3DGravityCurrent._fields_})


class F3DLogRecord(C.Structure):
    _fields_ = [
        ("iiter", C.c_int), ("time", C.c_double), ("dt", C.c_double), ("dtc", C.c_double),
        ("massvol", C.c_double), ("massdep", C.c_double), ("massdry", C.c_double),
        ("masswet", C.c_double), ("outmass", C.c_double), ("erumass", C.c_double),
    ]


LOG_FIELDS = [f for f, _ in F3DLogRecord._fields_]


def dptr(a):
    """Pointer to a C-contiguous float64 numpy array (or NULL for None)."""
    if a is None:
        return c_double_p()
    assert a.dtype == np.float64 and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(c_double_p)


def iptr(a):
    if a is None:
        return c_int_p()
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(c_int_p)


class Pinned:
    """Holds a ctypes struct together with the arrays it points into."""

    def __init__(self, struct, keep):
        self.struct = struct
        self._keep = keep

    def ref(self):
        return C.byref(self.struct)


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def make_grid(g: dict, precision: int = 64) -> Pinned:
    keep = {k: _f64(g[k]) for k in ("dz", "zlayer", "Hm1", "topg", "diam", "rhop", "psi", "sphe")}
    s = F3DGrid(
        nx=g["nx"], ny=g["ny"], nz=g["nz"], nc=g["nc"], np=g["np"], coord_sys=g["coord_sys"],
        modkv=g["modkv"], modkh=g["modkh"], modv=g["modv"], wetdep=g["wetdep"],
        aggregate=g["aggregate"], precision=precision, dX1=g["dX1"], dX2=g["dX2"], dx=g["dx"],
        dy=g["dy"], rkh0=g["rkh0"], rkv0=g["rkv0"], Csh=g["Csh"], safety_factor=g["safety_factor"],
        vset_factor=g["vset_factor"],
        dz=dptr(keep["dz"]), zlayer=dptr(keep["zlayer"]), Hm1=dptr(keep["Hm1"]),
        topg=dptr(keep["topg"]), diam=dptr(keep["diam"]), rhop=dptr(keep["rhop"]),
        psi=dptr(keep["psi"]), sphe=dptr(keep["sphe"]))
    return Pinned(s, keep)


def make_met(m: dict, agg: dict = None) -> Pinned:
    """f3d_met_series of a met dict; agg (synth.aggregation_inputs) adds the
    QV and P snapshots of the aggregation model."""
    keep = {k: _f64(m[k]) for k in ("u", "v", "w", "t", "tp", "rho", "ust", "pblh", "rmol", "znt",
                                     "prate", "ldu")}
    keep["times"] = _i32(m["times"])
    extra = {}
    if agg is not None:
        keep["qv"], keep["p"] = _f64(agg["qv"]), _f64(agg["p"])
        extra = dict(qv=dptr(keep["qv"]), p=dptr(keep["p"]))
    s = F3DMetSeries(nt=len(keep["times"]), times=iptr(keep["times"]), time_lag=float(m["time_lag"]),
                     **{k: dptr(keep[k]) for k in ("u", "v", "w", "t", "tp", "rho", "ust", "pblh",
                                                   "rmol", "znt", "prate", "ldu")}, **extra)
    return Pinned(s, keep)


def make_src(sr: dict, agg: dict = None) -> Pinned:
    """f3d_src_series of a source dict; agg (synth.aggregation_inputs) adds
    the plume temperature lists of the intervals."""
    keep = {k: _i32(sr[k]) for k in ("t1", "t2", "nsou", "isrc", "jsrc", "ksrc")}
    keep["tmrat"] = _f64(sr["tmrat"])
    extra = {}
    if agg is not None:
        pl = agg["plume"]
        keep["nplume"] = _i32([len(q["ix"]) for q in pl])
        for k, f in (("pix", "ix"), ("piy", "iy"), ("piz", "iz")):
            keep[k] = _i32(np.concatenate([np.asarray(q[f]) for q in pl]) if pl else [])
        keep["ptemp"] = _f64(np.concatenate([np.asarray(q["t"]) for q in pl]) if pl else [])
        keep["pwater"] = _f64(np.concatenate([np.asarray(q["w"]) for q in pl]) if pl else [])
        extra = dict(nplume=iptr(keep["nplume"]), pix=iptr(keep["pix"]), piy=iptr(keep["piy"]),
                     piz=iptr(keep["piz"]), ptemp=dptr(keep["ptemp"]), pwater=dptr(keep["pwater"]))
    s = F3DSrcSeries(nint=len(keep["t1"]), tmrat=dptr(keep["tmrat"]),
                     **{k: iptr(keep[k]) for k in ("t1", "t2", "nsou", "isrc", "jsrc", "ksrc")}, **extra)
    return Pinned(s, keep)


def log_array(recs, n):
    return {f: np.array([getattr(recs[i], f) for i in range(n)]) for f in LOG_FIELDS}
