"""The gravity current (f3d_set_gravity_current: addradialwind at every
meteo update, divcorr at the mass-budget log steps) through the CUDA context
against the oracle, whose restatement is pinned bit for bit to the
reference's own Fortran (tests/golden/small_gravity_current.npz).

Plain FP64 form: the radial wind is added to exactly the same cells and
levels (bitwise vx, vy after the first update), and the whole run agrees to
1e-12 as the runs without it do.  Precision form: the tile shapes agree bit
for bit, the binary64 form's column load within 1e-4."""
import numpy as np
import pytest

import fall3d_gb300 as F
import oracle_lib as O
from fall3d_gb300 import synth
from helpers import assert_close, assert_same_bits

pytestmark = pytest.mark.gpu

OVER = dict(M0=1e7, u10=4.0, vy0=1.0, run_h=0.75)


def _scen():
    return synth.make_scenario("small", seed=6, **OVER)


def test_radial_wind_added_like_the_oracle():
    s = _scen()
    gc = synth.gravity_current(s)
    o = O.OracleCtx(s)
    o.set_gravity_current(gc)
    g = F.Context(s, F.PREC_FP64)
    g.set_gravity_current(gc)
    for h in (o, g):
        h.source(0)
        h.meteo(0)
    co, cg = o.coeffs(), g.coeffs()
    # the reference's winds (and so the cells that change) are identical
    # bit for bit before the radial wind: compare where it acted as well
    g0 = F.Context(s, F.PREC_FP64)
    g0.source(0)
    g0.meteo(0)
    changed = cg["vx"] != g0.coeffs()["vx"]
    assert changed.sum() > 10
    for k in ("vx", "vy"):
        assert_same_bits(cg[k], co[k], k)
    assert_close(np.array([g.state()["dt"]]), np.array([o.state()["dt"]]), 1e-14, 0.0, "dt")


def test_run_fp64_with_gravity_current():
    s = _scen()
    gc = synth.gravity_current(s)
    o = O.OracleCtx(s, nthreads=8)
    o.set_gravity_current(gc)
    lo = o.run()
    g = F.Context(s, F.PREC_FP64)
    g.set_gravity_current(gc)
    lg = g.run()
    assert g.state()["iiter"] == o.state()["iiter"]
    assert np.array_equal(lg["iiter"], lo["iiter"])
    for k in ("time", "dt"):
        assert_close(lg[k], lo[k], 1e-14, 0.0, k)
    for k in ("massvol", "massdep", "outmass"):
        assert_close(lg[k], lo[k], 1e-12, 0.0, k)
    fo, fg = o.fields(), g.fields()
    assert_close(fg["c"], fo["c"], 1e-12, 1e-9, "c")
    assert_close(fg["cdry"], fo["cdry"], 1e-12, 1e-9, "cdry")
    # the correction acts: the run differs from one without the current
    g0 = F.Context(s, F.PREC_FP64)
    g0.run()
    assert not np.array_equal(g0.fields()["c"], fg["c"])


def test_fp32_with_gravity_current():
    """Precision form: every tile shape of the fused step agrees bit for
    bit, the per-routine binary32 path within its reciprocal-vs-divide
    1e-5, and the column load of the binary64 form within 1e-4."""
    s = _scen()
    gc = synth.gravity_current(s)
    res = {}
    for name, prec, fused, tile in (("t0", F.PREC_FP32, 1, 0), ("t3", F.PREC_FP32, 1, 3),
                                    ("per", F.PREC_FP32, 0, 0), ("fp64", F.PREC_FP64, 0, 0)):
        g = F.Context(s, prec)
        if prec == F.PREC_FP32:
            g.set_option(F.OPT_FUSED, fused)
            g.set_option(F.OPT_TILE, tile)
        g.set_gravity_current(gc)
        log = g.run()
        res[name] = (g.fields(), log, g.outputs())
    for k in ("c", "cdry", "cwet"):
        assert_same_bits(res["t3"][0][k], res["t0"][0][k], k)
    assert np.array_equal(res["t3"][1]["iiter"], res["fp64"][1]["iiter"])
    for k in ("load", "col_mass"):
        ref = res["per"][2][k]
        assert np.max(np.abs(res["t3"][2][k] - ref)) <= 1e-5 * np.max(np.abs(ref)), k
        ref = res["fp64"][2][k]
        assert np.max(np.abs(res["t3"][2][k] - ref)) <= 1e-4 * np.max(np.abs(ref)), k


def test_gravity_current_rejected_in_batch():
    s = _scen()
    g = F.Context(s, F.PREC_FP32)
    g.set_gravity_current(synth.gravity_current(s))
    b = F.Batch(2)
    with pytest.raises(F.F3DError):
        b.add(g)
    b.close()
    g.set_gravity_current(None)


def test_wind_output_with_gravity_current():
    """The gravity-current wind variables of printres_nc.f90:603-644:
    vx*Hm1 and vy*Hm1 on the levels, and moved to heights above sea level
    by ter2asl (the oracle's ter2asl, pinned to the reference's)."""
    s = _scen()
    g = F.Context(s, F.PREC_FP64)
    g.set_gravity_current(synth.gravity_current(s))
    g.source(0)
    g.meteo(0)
    co = g.coeffs()
    hm = np.asarray(s.grid["Hm1"])
    lib = O.load()
    nz, ny, nx = co["vx"].shape
    for index, key in ((1, "vx"), (2, "vy")):
        want = co[key] * hm[None]
        assert_same_bits(g.output(F.OUT_WIND, index), want, key)
        asl = np.ascontiguousarray(want.copy())
        lib.orc_ter2asl(O.p(asl), O.p(np.ascontiguousarray(s.grid["topg"], dtype=np.float64)),
                        O.p(np.ascontiguousarray(s.grid["zlayer"], dtype=np.float64)), nx, ny, nz)
        assert_same_bits(g.output(F.OUT_WIND, index, asl=True), asl, key + " asl")
