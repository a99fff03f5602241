"""Driver of the translated reference (oracle/_ref/libf3dref.so) -- test
infrastructure: the golden fixtures (tests/golden/make_golden.py) and the
CPU baseline of bench.py run the reference's own Fortran through it.

The library is the reference's Sources/*.f90 translated to C by
oracle/ref_translate.py; its module variables are exported as ``m_<name>``
and its subroutines as ``f90_<name>``.  What the driver does itself, because
those lines of the reference read files: it puts each DBS snapshot into the
Master arrays and applies the two post-read operations of Sources/reamet.f90
(PRATE*3600 when wet deposition is on, vz(:,:,1)=0), and it puts each source
interval into the arrays that Sources/reasrc.f90 fills.  Everything else
(meteo, kappa3, setvset, setvdrydep, scaling, corvver, setdivu, finddt,
source, setsrc, sizloop with all its routines, getc0, cmass3d) is the
reference's code, stepped by the time loop of Sources/Fall3d.f90:73-121.

``RefRun(scen, ic_loc=, nc_loc=)`` restricts the class loops to a range of
classes, as one rank of the reference's class decomposition
(Sources/Domain.f90 ic_loc / nc_loc; sizloop.f90:31, setsrc.f90:50,
cmass2d.f90:42): ``time_steps`` times such a rank, and bench.py runs one per
host core to time the reference's class-parallel run.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import shutil
import time as _time

import numpy as np


class RefLib:
    """One fresh load of the translated reference: a program run starts with
    its SAVE variables at their initial values (vsettl's cd = 1, the first-call
    set-up of setvdrydep and cmass2d), so each run gets its own copy."""

    _n = 0

    def __init__(self):
        import ref_translate

        src = ref_translate.build()
        RefLib._n += 1
        path = src.replace(".so", f".run{os.getpid()}_{RefLib._n}.so")
        shutil.copyfile(src, path)
        self.lib = C.CDLL(path)
        os.unlink(path)

    def i(self, name):
        return C.c_int.in_dll(self.lib, "m_" + name)

    def d(self, name):
        return C.c_double.in_dll(self.lib, "m_" + name)

    def arr(self, name, n, ctype=C.c_double):
        ptr = C.c_void_p.in_dll(self.lib, "m_" + name).value
        assert ptr, name
        return np.ctypeslib.as_array((ctype * n).from_address(ptr))

    def fixed(self, name, n, ctype=C.c_double):
        return np.ctypeslib.as_array((ctype * n).in_dll(self.lib, "m_" + name))

    def setstr(self, name, value, length):
        buf = (C.c_char * (length + 1)).in_dll(self.lib, "m_" + name)
        v = value.encode().ljust(length)[:length]
        C.memmove(buf, v + b"\0", length + 1)

    def call(self, name, *args):
        f = getattr(self.lib, "f90_" + name)
        f.restype = None
        f(*args)

    def ptr(self, name):
        return C.c_void_p(C.c_void_p.in_dll(self.lib, "m_" + name).value)


def iaggr_of(diam, np_):
    """Index of the first aggregating class (readat.f90:400-409): the lowest
    class finer than the aggregate class np, else np-1."""
    iaggr = 0
    for ic in range(np_ - 1, 0, -1):
        if diam[np_ - 1] > diam[ic - 1]:
            iaggr = ic
    return iaggr if iaggr else np_ - 1


class RefRun:
    """The reference's set-up (readat / reagrd / getmem1 of Sources/setup.f90)
    for a synthetic scenario; gc: GRAVITY_CURRENT parameters
    (synth.gravity_current) or None; agg: aggregation inputs
    (synth.aggregation_inputs) or None; ic_loc / nc_loc: the class range this
    run steps (1-based, all classes by default)."""

    def __init__(self, scen, gc=None, agg=None, ic_loc=1, nc_loc=None):
        self.R = R = RefLib()
        self.scen, self.gc, self.agg = scen, gc, agg
        g = scen.grid
        nx, ny, nz, nc = g["nx"], g["ny"], g["nz"], g["nc"]
        self.dims = (nx, ny, nz, nc)
        nc_loc = nc if nc_loc is None else nc_loc
        for k, v in (("nx", nx), ("ny", ny), ("nz", nz), ("nc", nc), ("np", g["np"]), ("ng", nc - g["np"]),
                     ("modkv", g["modkv"]), ("modkh", g["modkh"]), ("modv", g["modv"]), ("lmeth", 1),
                     ("nz_loc", nz), ("nc_loc", nc_loc), ("iz_loc", 1), ("ic_loc", ic_loc), ("iiter", 0),
                     ("wetdeposition", g["wetdep"]), ("aggregation", 1 if agg else 0), ("gravity_current", 0),
                     ("meteotime", 1), ("sourcetime", 1)):
            R.i(k).value = int(v)
        for k, v in (("dx1", g["dX1"]), ("dx2", g["dX2"]), ("dx", g["dx"]), ("dy", g["dy"]),
                     ("csh", g["Csh"]), ("rkh0", g["rkh0"]), ("rkv0", g["rkv0"]),
                     ("safety_factor", g["safety_factor"]), ("vset_factor", g["vset_factor"]),
                     ("dt", 1.0), ("outmass", 0.0), ("erumass", 0.0)):
            R.d(k).value = float(v)
        R.setstr("coord_sys", "LON-LAT" if g["coord_sys"] == 0 else "UTM", 10)
        if gc:  # readat.f90:150-213, reagrd.f90:152-153
            R.i("gravity_current").value = 1
            for k in ("c_flow_rate", "lambda_grav", "k_entrain", "brunt_vaisala"):
                R.d(k).value = gc[k]
            for k in ("radial_wind_lon", "radial_wind_x"):
                R.d(k).value = gc["center_x"]
            for k in ("radial_wind_lat", "radial_wind_y"):
                R.d(k).value = gc["center_y"]
            R.d("xorigr").value = gc["xorigr"]
            R.d("yorigr").value = gc["yorigr"]
            R.d("beg_time").value = gc["beg_time"]
        names = (C.c_char * 26 * 50).in_dll(R.lib, "m_classname")
        for ic in range(50):
            C.memmove(names[ic], b" " * 25 + b"\0", 26)
        for k in ("diam", "rhop", "psi", "sphe"):
            R.fixed(k, 50)[:nc] = g[k]
        if g.get("aggregate"):  # classname(np) == 'aggregate' (setvset.f90:48)
            C.memmove(names[g["np"] - 1], b"aggregate".ljust(25) + b"\0", 26)
        if agg:  # readat_aggr (readat.f90:350-440)
            R.i("iaggr").value = iaggr_of(list(g["diam"]), g["np"])
            R.d("df").value = agg["Df"]
            R.i("ndtagr").value = agg["ndtagr"]
            R.fixed("fc", 50)[:g["np"]] = agg["fc"]
        R.call("getmem1")
        pl, s3 = nx * ny, nx * ny * nz
        self.pl, self.s3 = pl, s3
        R.arr("hm1", pl)[:] = np.asarray(g["Hm1"]).ravel()
        R.arr("zlayer", nz)[:] = g["zlayer"]
        R.arr("dz", nz + 1)[:] = g["dz"]
        R.arr("topg", pl)[:] = np.asarray(g["topg"]).ravel()
        R.arr("ldu", pl)[:] = np.asarray(scen.met["ldu"]).ravel()
        self.src_alloc = False
        R.d("time").value = scen.beg_time

    def meteo(self, it):
        """The DBS snapshot it into the Master arrays (reamet.f90), then meteo."""
        R, m, g, s3, pl = self.R, self.scen.met, self.scen.grid, self.s3, self.pl
        for k, f in (("vx", "u"), ("vy", "v"), ("vz", "w"), ("tempe", "t"), ("vptemp", "tp"),
                     ("rho", "rho")):
            R.arr(k, s3)[:] = m[f][it].ravel()
        for k, f in (("ustar", "ust"), ("zi", "pblh"), ("rl", "rmol"), ("znt", "znt")):
            R.arr(k, pl)[:] = m[f][it].ravel()
        if g["wetdep"]:
            pr = R.arr("prate", pl)
            pr[:] = m["prate"][it].ravel()
            pr[:] = pr * 3600.0  # reamet.f90:146
        R.arr("vz", s3)[:pl] = 0.0  # reamet.f90:153
        if self.agg:  # the DBS variables QV and P
            R.arr("qv", s3)[:] = self.agg["qv"][it].ravel()
            R.arr("p", s3)[:] = self.agg["p"][it].ravel()
        R.call("meteo")

    def source(self, iint):
        """Source interval iint into the arrays reasrc.f90 fills, then source."""
        R, sr, nc, s3 = self.R, self.scen.src, self.dims[3], self.s3
        nx, ny = self.dims[0], self.dims[1]
        off = int(np.sum(sr["nsou"][:iint]))
        n = int(sr["nsou"][iint])
        if self.src_alloc:
            R.call("outmem2")
        R.i("nsou").value = n
        R.call("getmem2")
        self.src_alloc = True
        if n:
            R.arr("isrc", n, C.c_int)[:] = sr["isrc"][off:off + n]
            R.arr("jsrc", n, C.c_int)[:] = sr["jsrc"][off:off + n]
            R.arr("ksrc", n, C.c_int)[:] = sr["ksrc"][off:off + n]
            R.arr("tmrat", n * nc)[:] = sr["tmrat"][off * nc:(off + n) * nc]
            if self.gc:  # the source points' heights (get_source_coordinates)
                R.arr("zs", n)[:] = np.full(n, self.gc["h_tot"]) if iint else self.scen.info["zs"][:n]
        R.call("source")
        if self.agg:  # settemplume (source.f90:89-149) from the plume file
            tp, wp = R.arr("tplume", s3), R.arr("wplume", s3)
            tp[:] = 0.0
            wp[:] = 0.0
            pl_ = self.agg["plume"][iint]
            for q in range(len(pl_["ix"])):
                cell = (pl_["ix"][q] - 1) + nx * (pl_["iy"][q] - 1) + nx * ny * (pl_["iz"][q] - 1)
                tp[cell] = pl_["t"][q]
                wp[cell] = pl_["w"][q]

    def step(self):
        """Fall3d.f90:112-117: time, iiter and erumass advance, setsrc, sizloop."""
        R = self.R
        dt = R.d("dt").value
        R.d("time").value = R.d("time").value + dt
        R.i("iiter").value = R.i("iiter").value + 1
        R.d("erumass").value = R.d("erumass").value + R.d("flowrate").value * dt
        R.call("setsrc")
        R.call("sizloop")
        return dt

    def budget(self):
        """getc0, cload = cdry + cwet and cmass3d (endstep.f90:35-60):
        (massvol, massdep, massdry, masswet)."""
        R = self.R
        nx, ny, nz, nc = self.dims
        pl = self.pl
        R.call("getc0")
        cl = R.arr("cload", pl * (nc + 1))
        cl[:] = R.arr("cdry", pl * (nc + 1)) + R.arr("cwet", pl * (nc + 1))
        out = [C.c_double() for _ in range(4)]
        dims = [C.c_int(v) for v in (nx, ny, nz, nc)]
        f = R.lib.f90_cmass3d
        f.restype = None
        f(R.ptr("c"), R.ptr("cload"), R.ptr("cdry"), R.ptr("cwet"), *[C.byref(x) for x in dims],
          C.byref(R.d("dx1")), C.byref(R.d("dx2")), R.ptr("dz"), *[C.byref(x) for x in out])
        return tuple(x.value for x in out)


def run(scen, max_steps=None, gc=None, agg=None):
    """The Fall3d.f90 loop on the translated reference; returns a dict of the
    final state, the mass-budget log (every 600 s, endstep.f90:51) and the
    coefficient fields after the first meteo update."""
    r = RefRun(scen, gc, agg)
    R, m, sr = r.R, scen.met, scen.src
    nx, ny, nz, nc = r.dims
    pl, s3 = r.pl, r.s3
    beg, end = scen.beg_time, scen.end_time
    meteo_time, source_time = beg, beg
    meteotime, sourcetime = True, True
    log = {k: [] for k in ("iiter", "time", "dt", "dtc", "massvol", "massdep", "massdry", "masswet",
                           "outmass", "erumass")}
    coeffs = None
    steps = 0
    hb = (nx + 2) * (ny + 2) * (nz + 2)
    while True:
        time = R.d("time").value
        aggregationtime = False
        if source_time <= time:
            if sourcetime:
                ts = int(time)
                it = next(i for i in range(len(sr["t1"])) if sr["t1"][i] <= ts < sr["t2"][i])
                r.source(it)
                aggregationtime = bool(agg)
                source_time = float(sr["t2"][it])
            if source_time >= end:
                sourcetime = False
        if meteo_time <= time:
            if meteotime:
                ts = int(m["time_lag"] + time)
                times = m["times"]
                itime, endsec = len(times) - 1, times[-1]
                for i in range(len(times) - 1):
                    if times[i] <= ts < times[i + 1]:
                        itime, endsec = i, times[i + 1]
                r.meteo(itime)
                aggregationtime = bool(agg)
                meteo_time = float(endsec) - m["time_lag"]
                if coeffs is None:
                    coeffs = {k: R.arr(k, s3).copy() for k in ("vx", "vy", "vz", "rho", "rkhor", "rkh1",
                                                                "rkver")}
                    coeffs["vset"] = R.arr("vset", s3 * nc).copy()
                    coeffs["vdep"] = R.arr("vdep", pl * nc).copy()
                    coeffs["dt"] = R.d("dt").value
            if meteo_time >= end:
                meteotime = False
        if aggregationtime:  # Fall3d.f90:101-110
            R.call("agrpar")
        dt = r.step()
        steps += 1
        time = R.d("time").value
        iiter = R.i("iiter").value
        if iiter == 1 or math.fmod(time, 600.0) <= dt:  # endstep.f90:51
            mv, md, mdry, mwet = r.budget()
            for k, v in (("iiter", iiter), ("time", time), ("dt", dt), ("dtc", R.d("dtc").value),
                         ("massvol", mv), ("massdep", md), ("massdry", mdry), ("masswet", mwet),
                         ("outmass", R.d("outmass").value), ("erumass", R.d("erumass").value)):
                log[k].append(v)
            if gc:  # endstep.f90:71, after writim
                R.d("massvol").value = mv
                R.d("massdep").value = md
                R.call("divcorr")
        if time >= end or (max_steps and steps >= max_steps):
            break
    res = {"c": R.arr("c", hb * nc).copy().reshape(nc, nz + 2, ny + 2, nx + 2),
           "cdry": R.arr("cdry", pl * (nc + 1)).copy().reshape(nc + 1, ny, nx),
           "cwet": R.arr("cwet", pl * (nc + 1)).copy().reshape(nc + 1, ny, nx),
           "iiter": R.i("iiter").value, "time": R.d("time").value, "dt": R.d("dt").value,
           "erumass": R.d("erumass").value, "outmass": R.d("outmass").value,
           "flowrate": R.d("flowrate").value}
    if agg:
        res["maggr"] = R.arr("maggr", s3).copy().reshape(nz, ny, nx)
    for k, v in log.items():
        res["log_" + k] = np.array(v)
    for k, v in coeffs.items():
        res["coef_" + k] = np.array(v)
    return res


def time_steps(scen, steps, ic_loc=1, nc_loc=None, warm=1, budget_s=None):
    """One rank of the reference's class decomposition on scen: the first
    source and meteo update (timed apart), ``warm`` untimed steps, then up to
    ``steps`` timed steps (setsrc + sizloop over classes ic_loc ..
    ic_loc+nc_loc-1), stopping early once budget_s seconds have passed.
    Returns (steps timed, seconds, meteo seconds, classes stepped)."""
    r = RefRun(scen, ic_loc=ic_loc, nc_loc=nc_loc)
    r.source(0)
    t0 = _time.perf_counter()
    r.meteo(0)
    t_met = _time.perf_counter() - t0
    for _ in range(warm):
        r.step()
    done = 0
    t0 = _time.perf_counter()
    while done < steps:
        r.step()
        done += 1
        if budget_s is not None and _time.perf_counter() - t0 > budget_s:
            break
    return done, _time.perf_counter() - t0, t_met, r.R.i("nc_loc").value


def class_groups(nc, ngrp):
    """(ic_loc, nc_loc) of each of ngrp class groups: Sources/Parallel.F90
    localdim (:189-211, the first nc mod ngrp groups take one class more)
    and globalindex (:165-185, the running offset)."""
    q, r = divmod(nc, ngrp)
    out, ic = [], 1
    for me in range(ngrp):
        n = q + 1 if me < r else q
        out.append((ic, n))
        ic += n
    return out


def time_class_parallel(scen, ngrp, steps, serial_steps=2, budget_s=30.0):
    """The reference's class-parallel run on ngrp host cores, without MPI:
    one process sets up the run (source, the first meteo update), times
    ``serial_steps`` steps over every class (the serial build), then forks
    one process per class group (Sources/Domain.f90:31-32), each stepping its
    classes after one untimed step; all start together and the wall time
    until the last one finishes is the parallel time.  The step count per
    group is min(steps, what fits budget_s at the serial per-class rate).
    Classes are independent within a step, so the groups need no exchange
    (the budget reductions of the MPI build are not timed).

    Returns a dict: meteo_s, serial (steps, seconds, cell_class_steps),
    parallel (groups, steps, seconds, cell_class_steps)."""
    import struct

    r = RefRun(scen)
    nx, ny, nz, nc = r.dims
    cells = nx * ny * nz
    r.source(0)
    t0 = _time.perf_counter()
    r.meteo(0)
    t_met = _time.perf_counter() - t0
    r.step()  # untimed
    t0 = _time.perf_counter()
    for _ in range(serial_steps):
        r.step()
    t_ser = _time.perf_counter() - t0
    groups = class_groups(nc, ngrp)
    per_class = t_ser / serial_steps / nc
    n_steps = int(max(2, min(steps, budget_s / (per_class * max(n for _, n in groups)))))
    go_r, go_w = os.pipe()
    kids = []
    for ic_loc, nc_loc in groups:
        rd, wr = os.pipe()
        pid = os.fork()
        if pid == 0:  # one class group
            code = 1
            try:
                os.close(rd)
                os.close(go_w)
                r.R.i("ic_loc").value = ic_loc
                r.R.i("nc_loc").value = nc_loc
                r.step()
                os.write(wr, b"r")
                os.read(go_r, 1)
                t = _time.perf_counter()
                for _ in range(n_steps):
                    r.step()
                os.write(wr, struct.pack("d", _time.perf_counter() - t))
                code = 0
            finally:
                os._exit(code)
        os.close(wr)
        kids.append((pid, rd))
    os.close(go_r)
    try:
        for _, rd in kids:
            if os.read(rd, 1) != b"r":
                raise RuntimeError("a class group failed before its timed steps")
        t0 = _time.perf_counter()
        os.write(go_w, b"g" * len(kids))
        own = []
        for _, rd in kids:
            b = os.read(rd, 8)
            if len(b) != 8:
                raise RuntimeError("a class group failed during its timed steps")
            own.append(struct.unpack("d", b)[0])
        t_par = _time.perf_counter() - t0
    finally:
        os.close(go_w)
        for pid, rd in kids:
            os.close(rd)
            os.waitpid(pid, 0)
    return {"meteo_s": t_met,
            "serial": {"steps": serial_steps, "seconds": t_ser, "cell_class_steps": cells * nc * serial_steps},
            "parallel": {"groups": len(groups), "steps": n_steps, "seconds": t_par,
                         "slowest_group_s": max(own), "cell_class_steps": cells * nc * n_steps}}
