"""The CPU oracle against golden vectors produced by the reference's own
Fortran (tests/golden/make_golden.py: the reference's hot-path source,
translated to C by oracle/ref_translate.py, driven through the Fall3d.f90
time loop).  Agreement is bit for bit: concentrations, ground deposits, the
mass-budget log, the time and time-step sequences, the step count and the
coefficient fields after the first meteo update."""
import json
import os

import numpy as np
import pytest

import oracle_lib as O
from fall3d_gb300 import synth
from helpers import assert_same_bits

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = json.load(open(os.path.join(HERE, "cases.json")))


def _scenario(meta):
    s = synth.make_scenario(meta["workload"], seed=meta["seed"], **meta["overrides"])
    if meta.get("aggregation"):
        synth.add_gas_class(s)
    if s.grid["wetdep"]:
        band = np.linspace(0.0, 4.0, s.grid["nx"])[None, :] / 3600.0
        s.met["prate"][:] = np.asarray(band, np.float32).astype(np.float64)
    return s


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_golden(name):
    meta = CASES[name]
    g = np.load(os.path.join(HERE, f"{name}.npz"))
    stride = int(g["sample_stride"]) if "sample_stride" in g else 1
    s = _scenario(meta)
    o = O.OracleCtx(s, nthreads=4)
    if "gravity_current" in meta:
        o.set_gravity_current(meta["gravity_current"])
    if meta.get("aggregation"):
        o.set_aggregation(synth.aggregation_inputs(s))
    log = o.run(max_steps=meta["max_steps"] or 0)
    st = o.state()
    assert st["iiter"] == int(g["iiter"]) == meta["steps"]
    f = o.fields()
    assert_same_bits(f["c"].ravel()[::stride], g["c"].ravel(), "c")
    assert_same_bits(f["cdry"].ravel(), g["cdry"].ravel(), "cdry")
    assert_same_bits(f["cwet"].ravel(), g["cwet"].ravel(), "cwet")
    if "maggr" in g:
        assert_same_bits(o.maggr(), g["maggr"], "maggr")
    for k in ("time", "dt", "erumass", "outmass", "flowrate"):
        assert_same_bits(np.array([st[k]]), np.array([float(g[k])]), k)
    for k in ("iiter", "time", "dt", "dtc", "massvol", "massdep", "massdry", "masswet", "outmass",
              "erumass"):
        assert_same_bits(np.asarray(log[k], float), np.asarray(g["log_" + k], float), "log " + k)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_coefficients_match_reference_golden(name):
    meta = CASES[name]
    g = np.load(os.path.join(HERE, f"{name}.npz"))
    stride = int(g["sample_stride"]) if "sample_stride" in g else 1
    s = _scenario(meta)
    o = O.OracleCtx(s)
    if "gravity_current" in meta:
        o.set_gravity_current(meta["gravity_current"])
    o.source(0)
    o.meteo(0)
    co = o.coeffs()
    f = o.fields()
    for k in ("vx", "vy", "vz", "rho", "rkhor", "rkh1", "rkver"):
        assert_same_bits(co[k].ravel()[::stride], g["coef_" + k].ravel(), k)
    assert_same_bits(f["vset"].ravel()[::stride], g["coef_vset"].ravel(), "vset")
    assert_same_bits(f["vdep"].ravel(), g["coef_vdep"].ravel(), "vdep")
    assert o.state()["dt"] == float(g["coef_dt"])


def test_output_cuts_match_reference_golden():
    """Flight-level cuts (setcut_FL with standard_atm) and the terrain-following
    to sea-level conversion (ter2asl) of the oracle against the reference's
    own Fortran of Sources/setcut.f90 and Sources/ter2asl.f90."""
    g = np.load(os.path.join(HERE, "output_cuts.npz"))
    lib = O.load()
    nz, ny, nx = g["var3d"].shape
    zl, topg = np.ascontiguousarray(g["zlayer"]), np.ascontiguousarray(g["topg"])
    var3d, pres = np.ascontiguousarray(g["var3d"]), np.ascontiguousarray(g["pres"])
    for n, fl in enumerate(g["fls"]):
        out = np.zeros((ny, nx))
        lib.orc_setcut_fl(nx, ny, nz, O.p(out), O.p(var3d), O.p(pres), float(fl) * 30.48)
        assert_same_bits(out, g["cut"][n], f"FL{fl:g}")
    patm = np.array([lib.orc_standard_pressure(float(z)) for z in g["zs"]])
    assert_same_bits(patm, g["patm"], "standard_atm")
    conc = np.array(g["conc"])
    lib.orc_ter2asl(O.p(conc), O.p(topg), O.p(zl), nx, ny, nz)
    assert_same_bits(conc, g["asl"], "ter2asl")
