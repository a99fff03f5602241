"""Generates the golden vectors in tests/golden/ from the reference's own
Fortran source.

    python tests/golden/make_golden.py

oracle/ref_translate.py translates the reference's hot-path Fortran (its
Sources/ directory) into C and compiles it into oracle/_ref/.  This
script drives that library through the time loop of Sources/Fall3d.f90:73-121
on seeded synthetic scenarios and stores its state (concentrations, deposits,
the mass-budget log, the coefficient fields after the first meteo update) as
compressed fixtures.  It needs the reference sources and so runs only where
they are mounted; the fixtures it writes are committed.

What the driver does itself, because those lines of the reference read
files: it puts each DBS snapshot into the Master arrays and applies the two
post-read operations of Sources/reamet.f90 (PRATE*3600 when wet deposition is
on, vz(:,:,1)=0), and it puts each source interval into the arrays that
Sources/reasrc.f90 fills.  Everything else (meteo, kappa3, setvset, setvdrydep,
scaling, corvver, setdivu, finddt, source, setsrc, sizloop with all its
routines, getc0, cmass3d) is the reference's code.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from fall3d_gb300 import synth  # noqa: E402

# (fixture name, workload, seed, overrides, max steps or None for the full run)
CASES = [
    ("tiny_similarity_rams", "tiny", 1, {}, None),
    ("small_wet", "small", 2, dict(wetdep=True, run_h=0.5), None),
    ("small_constant_cmaq_arastoopour", "small", 3,
     dict(modkv=0, modkh=2, modv=1, rkv0=35.0, rkh0=500.0, run_h=0.5), None),
    ("tiny_surface_wilson_utm", "tiny", 4,
     dict(modkv=2, modkh=1, modv=3, coord=1, spacing=4000.0, rmol=-1.0 / 300.0), None),
    ("tiny_dellino_ganser_two_updates", "tiny", 5, dict(modv=4, run_h=1.5, met_dt_h=0.5), None),
    ("cfg0_first_60_steps", "cfg0", 0, {}, 60),
    ("small_gravity_current", "small", 6, dict(M0=1e7, u10=4.0, vy0=1.0, run_h=0.75), None),
    ("small_aggregation", "small", 9, dict(nc=7, phimin=3.0, phimax=8.0, aggregate=[0.2, 1000.0, 0.2],
                                           M0=1e7, run_h=0.75), None),
]
# cases run with GRAVITY_CURRENT = YES (parameters of synth.gravity_current)
GRAVITY = {"small_gravity_current"}
# cases run with aggregation in transport: a gas class appended
# (synth.add_gas_class) and the inputs of synth.aggregation_inputs
AGGREGATION = {"small_aggregation"}
# large cases keep every SAMPLE-th value of the 3-D/4-D fields
SAMPLE = {"cfg0_first_60_steps": 37}


class RefLib:
    """One fresh load of the translated reference: a program run starts with
    its SAVE variables at their initial values (vsettl's cd = 1, the first-call
    set-up of setvdrydep and cmass2d), so each case gets its own copy."""

    _n = 0

    def __init__(self):
        import shutil
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


def iaggr_of(diam, np_):
    """Index of the first aggregating class (readat.f90:400-409): the lowest
    class finer than the aggregate class np, else np-1."""
    iaggr = 0
    for ic in range(np_ - 1, 0, -1):
        if diam[np_ - 1] > diam[ic - 1]:
            iaggr = ic
    return iaggr if iaggr else np_ - 1


def run_reference(scen, max_steps=None, gc=None, agg=None):
    """The Fall3d.f90 loop on the translated reference; returns a dict.
    gc: GRAVITY_CURRENT parameters (synth.gravity_current) or None;
    agg: aggregation inputs (synth.aggregation_inputs) or None."""
    R = RefLib()
    g, m, sr = scen.grid, scen.met, scen.src
    nx, ny, nz, nc = g["nx"], g["ny"], g["nz"], g["nc"]
    for k, v in (("nx", nx), ("ny", ny), ("nz", nz), ("nc", nc), ("np", g["np"]), ("ng", nc - g["np"]),
                 ("modkv", g["modkv"]), ("modkh", g["modkh"]), ("modv", g["modv"]), ("lmeth", 1),
                 ("nz_loc", nz), ("nc_loc", nc), ("iz_loc", 1), ("ic_loc", 1), ("iiter", 0),
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
    R.arr("hm1", pl)[:] = np.asarray(g["Hm1"]).ravel()
    R.arr("zlayer", nz)[:] = g["zlayer"]
    R.arr("dz", nz + 1)[:] = g["dz"]
    R.arr("topg", pl)[:] = np.asarray(g["topg"]).ravel()
    R.arr("ldu", pl)[:] = np.asarray(m["ldu"]).ravel()

    def meteo(it):
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
        if agg:  # the DBS variables QV and P
            R.arr("qv", s3)[:] = agg["qv"][it].ravel()
            R.arr("p", s3)[:] = agg["p"][it].ravel()
        R.call("meteo")

    state = {"src_alloc": False}

    def source(iint):
        off = int(np.sum(sr["nsou"][:iint]))
        n = int(sr["nsou"][iint])
        if state["src_alloc"]:
            R.call("outmem2")
        R.i("nsou").value = n
        R.call("getmem2")
        state["src_alloc"] = True
        if n:
            R.arr("isrc", n, C.c_int)[:] = sr["isrc"][off:off + n]
            R.arr("jsrc", n, C.c_int)[:] = sr["jsrc"][off:off + n]
            R.arr("ksrc", n, C.c_int)[:] = sr["ksrc"][off:off + n]
            R.arr("tmrat", n * nc)[:] = sr["tmrat"][off * nc:(off + n) * nc]
            if gc:  # the source points' heights (get_source_coordinates)
                R.arr("zs", n)[:] = np.full(n, gc["h_tot"]) if iint else scen.info["zs"][:n]
        R.call("source")
        if agg:  # settemplume (source.f90:89-149) from the plume file
            tp, wp = R.arr("tplume", s3), R.arr("wplume", s3)
            tp[:] = 0.0
            wp[:] = 0.0
            pl_ = agg["plume"][iint]
            for q in range(len(pl_["ix"])):
                cell = (pl_["ix"][q] - 1) + nx * (pl_["iy"][q] - 1) + nx * ny * (pl_["iz"][q] - 1)
                tp[cell] = pl_["t"][q]
                wp[cell] = pl_["w"][q]

    beg, end = scen.beg_time, scen.end_time
    R.d("time").value = beg
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
                source(it)
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
                meteo(itime)
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
        dt = R.d("dt").value
        R.d("time").value = R.d("time").value + dt  # Fall3d.f90:112-114
        R.i("iiter").value = R.i("iiter").value + 1
        R.d("erumass").value = R.d("erumass").value + R.d("flowrate").value * dt
        R.call("setsrc")
        R.call("sizloop")
        steps += 1
        time = R.d("time").value
        iiter = R.i("iiter").value
        if iiter == 1 or math.fmod(time, 600.0) <= dt:  # endstep.f90:51
            R.call("getc0")
            cl = R.arr("cload", pl * (nc + 1))
            cl[:] = R.arr("cdry", pl * (nc + 1)) + R.arr("cwet", pl * (nc + 1))
            out = [C.c_double() for _ in range(4)]
            dims = [C.c_int(v) for v in (nx, ny, nz, nc)]
            f = R.lib.f90_cmass3d
            f.restype = None
            f(C.c_void_p(C.c_void_p.in_dll(R.lib, "m_c").value), C.c_void_p(C.c_void_p.in_dll(R.lib, "m_cload").value),
              C.c_void_p(C.c_void_p.in_dll(R.lib, "m_cdry").value), C.c_void_p(C.c_void_p.in_dll(R.lib, "m_cwet").value),
              *[C.byref(x) for x in dims], C.byref(R.d("dx1")), C.byref(R.d("dx2")),
              C.c_void_p(C.c_void_p.in_dll(R.lib, "m_dz").value), *[C.byref(x) for x in out])
            for k, v in (("iiter", iiter), ("time", time), ("dt", dt), ("dtc", R.d("dtc").value),
                         ("massvol", out[0].value), ("massdep", out[1].value),
                         ("massdry", out[2].value), ("masswet", out[3].value),
                         ("outmass", R.d("outmass").value), ("erumass", R.d("erumass").value)):
                log[k].append(v)
            if gc:  # endstep.f90:71, after writim
                R.d("massvol").value = out[0].value
                R.d("massdep").value = out[1].value
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


def scenario(workload, seed, over):
    s = synth.make_scenario(workload, seed=seed, **over)
    if s.grid["wetdep"]:
        band = np.linspace(0.0, 4.0, s.grid["nx"])[None, :] / 3600.0
        s.met["prate"][:] = np.asarray(band, np.float32).astype(np.float64)
    return s


def cuts():
    """Sources/setcut.f90 (setcut_FL, standard_atm) and Sources/ter2asl.f90
    of the translated reference on a seeded 9x7x12 case: heights around the
    three ICAO layers, topography below, at and above sea level, flight
    levels below the ground and above the top, and an unsorted-pressure
    column.  Stored in output_cuts.npz."""
    R = RefLib()
    rng = np.random.default_rng(7)
    nx, ny, nz = 9, 7, 12
    zl = np.concatenate([[0.0, 150.0, 400.0], np.linspace(800.0, 16000.0, nz - 3)])
    topg = rng.uniform(-200.0, 3000.0, (ny, nx))
    topg[0, 0], topg[0, 1], topg[1, 0] = 0.0, -50.0, 12000.0
    var3d = rng.uniform(0.0, 1.0, (nz, ny, nx))
    zabs = zl[:, None, None] + np.maximum(topg, 0.0)[None]
    _, pres, _ = synth.standard_atmosphere(zabs)
    pres = pres * (1.0 + 0.01 * rng.standard_normal(pres.shape))
    pres[:, 2, 3] = pres[::-1, 2, 3]  # increasing with height: no bracket
    pres = np.ascontiguousarray(pres)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    ni, nj, nk = C.c_int(nx), C.c_int(ny), C.c_int(nz)
    fls = np.array([0.0, 5.0, 50.0, 100.0, 200.0, 350.0, 450.0, 700.0, 1200.0])
    cut = np.zeros((len(fls), ny, nx))
    for n, fl in enumerate(fls):
        out = np.zeros((ny, nx))
        R.call("setcut_fl", C.byref(ni), C.byref(nj), C.byref(nk), dp(zl), dp(out), dp(var3d), dp(topg),
               dp(pres), C.byref(C.c_double(fl * 30.48)))
        cut[n] = out
    zs = np.array([-100.0, 0.0, 1524.0, 10999.0, 11000.0, 15000.0, 19999.5, 20000.0, 30000.0])
    patm = np.zeros(len(zs))
    for n, z in enumerate(zs):
        pp, tt = C.c_double(), C.c_double()
        R.call("standard_atm", C.byref(pp), C.byref(tt), C.byref(C.c_double(z)))
        patm[n] = pp.value
    conc = np.ascontiguousarray(rng.uniform(0.0, 1.0, (nz, ny, nx)))
    asl = conc.copy()
    R.call("ter2asl", dp(asl), dp(topg), dp(zl), C.byref(ni), C.byref(nj), C.byref(nk))
    path = os.path.join(HERE, "output_cuts.npz")
    np.savez_compressed(path, zlayer=zl, topg=topg, var3d=var3d, pres=pres, fls=fls, cut=cut, zs=zs,
                        patm=patm, conc=conc, asl=asl)
    print(f"output_cuts: {os.path.getsize(path) / 1024:.0f} KB")


def main():
    """All fixtures; --cuts only output_cuts.npz; --case NAME only that case
    (its cases.json entry replaced)."""
    if "--case" not in sys.argv:
        cuts()
    if "--cuts" in sys.argv:
        return
    only = sys.argv[sys.argv.index("--case") + 1] if "--case" in sys.argv else None
    meta = json.load(open(os.path.join(HERE, "cases.json"))) if only else {}
    for name, workload, seed, over, max_steps in CASES:
        if only and name != only:
            continue
        s = scenario(workload, seed, over)
        gc = synth.gravity_current(s) if name in GRAVITY else None
        agg = None
        if name in AGGREGATION:
            synth.add_gas_class(s)
            agg = synth.aggregation_inputs(s)
        r = run_reference(s, max_steps, gc, agg)
        path = os.path.join(HERE, f"{name}.npz")
        st = SAMPLE.get(name)
        if st:
            for k in ("c", "coef_vset", "coef_vx", "coef_vy", "coef_vz", "coef_rho", "coef_rkhor",
                      "coef_rkh1", "coef_rkver"):
                r[k] = np.asarray(r[k]).ravel()[::st].copy()
            r["sample_stride"] = st
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in r.items()})
        meta[name] = {"workload": workload, "seed": seed, "overrides": over, "max_steps": max_steps,
                      "steps": int(r["iiter"])}
        if gc:
            meta[name]["gravity_current"] = gc
        if agg:
            meta[name]["aggregation"] = True
        print(f"{name}: {r['iiter']} steps, {os.path.getsize(path) / 1024:.0f} KB")
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
