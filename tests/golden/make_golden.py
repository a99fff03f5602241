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

The driver (oracle/ref_driver.py) fills what the reference reads from
files (the DBS snapshots, the source intervals); everything else is the
reference's code.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from fall3d_gb300 import synth  # noqa: E402
from ref_driver import RefLib, run as run_reference  # noqa: E402

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
    ("cfg0_full_run", "cfg0", 0, {}, None),
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
SAMPLE = {"cfg0_first_60_steps": 37, "cfg0_full_run": 37}


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
