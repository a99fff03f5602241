"""The precision form's fused step kernel (f3d_fused.cu).

* Every tile shape computes each cell with the same operations, so all
  shapes agree bit for bit.
* Against the per-routine binary32 path (one kernel per reference routine)
  it differs only by reciprocal-multiply vs divide: 1e-5 relative.
* Against the binary64 plain form: identical step sequence, column load and
  ground deposit within 1e-4 (the precision-form target).
"""
import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import synth
from helpers import assert_same_bits

pytestmark = pytest.mark.gpu


def _run(s, prec, fused=1, tile=0, **kw):
    g = F.Context(s, prec)
    if prec == F.PREC_FP32:
        g.set_option(F.OPT_FUSED, fused)
        g.set_option(F.OPT_TILE, tile)
    log = g.run(**kw)
    return g, log


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("name,over", [("tiny", {}), ("small", dict(nx=61, ny=45, nz=9)),
                                       ("small", dict(wetdep=True)),
                                       ("small", dict(nx=150, ny=80, nz=12, wetdep=True))])
def test_tile_shapes_agree_bitwise(name, over):
    s = synth.make_scenario(name, seed=7, **over)
    if s.grid["wetdep"]:
        s.met["prate"][:] = np.float32(3.0 / 3600.0)
    res = []
    for tile in (0, 1, 2, 3):
        g, _ = _run(s, F.PREC_FP32, 1, tile, max_steps=12)
        f = g.fields()
        res.append((f["c"], f["cdry"], f["cwet"], g.state()["outmass"]))
    for r in res[1:]:
        assert_same_bits(r[0], res[0][0], "c")
        assert_same_bits(r[1], res[0][1], "cdry")
        assert_same_bits(r[2], res[0][2], "cwet")
        assert r[3] == res[0][3]


@pytest.mark.parametrize("wet", [False, True])
def test_fused_matches_per_routine_fp32(wet):
    s = synth.make_scenario("small", seed=8, wetdep=wet, run_h=1.0)
    if wet:
        s.met["prate"][:] = np.float32(2.0 / 3600.0)
    gf, lf = _run(s, F.PREC_FP32, 1)
    gu, lu = _run(s, F.PREC_FP32, 0)
    assert np.array_equal(lf["iiter"], lu["iiter"])
    of, ou = gf.outputs(), gu.outputs()
    for k in ("load", "col_mass", "c_grnd"):
        assert _rel(of[k], ou[k]) <= 1e-5, k
    ff, fu = gf.fields(), gu.fields()
    assert _rel(ff["cwet"], fu["cwet"] + 1e-300) <= 1e-5 if wet else True
    for k in ("massvol", "massdep", "outmass"):
        assert np.max(np.abs(lf[k] - lu[k]) / np.maximum(np.abs(lu[k]), 1e-300)) <= 1e-5, k


def test_fused_fp32_vs_fp64_cfg0():
    s = synth.make_scenario("cfg0", seed=0)
    g64, l64 = _run(s, F.PREC_FP64)
    g32, l32 = _run(s, F.PREC_FP32, 1)
    assert np.array_equal(l32["iiter"], l64["iiter"])
    assert_same_bits(l32["dt"], l64["dt"], "dt")
    o64, o32 = g64.outputs(), g32.outputs()
    for k in ("load", "col_mass"):
        assert _rel(o32[k], o64[k]) <= 1e-4, k
    tot64 = l64["massvol"] + l64["massdep"] + l64["outmass"]
    tot32 = l32["massvol"] + l32["massdep"] + l32["outmass"]
    assert np.max(np.abs(tot32 - tot64) / tot64) <= 1e-5


def test_fused_state_roundtrip():
    """Downloading and re-uploading the binary32 state continues identically."""
    s = synth.make_scenario("tiny", seed=9)
    a, _ = _run(s, F.PREC_FP32, 1, max_steps=20)
    b, _ = _run(s, F.PREC_FP32, 1, max_steps=10)
    st = b.state()
    f = b.fields()
    c = F.Context(s, F.PREC_FP32)
    c.source(0)
    c.meteo(0)
    c.upload_state(f["c"], f["cdry"], f["cwet"], st["erumass"], st["outmass"], st["cd"])
    c.set_time(st["time"], st["iiter"])
    for _ in range(10):
        c.step()
    assert_same_bits(c.fields()["c"], a.fields()["c"], "resumed")


@pytest.mark.parametrize("nz", [3, 4, 5])
def test_shallow_columns(nz):
    """The column march's first and last planes with no steady plane between
    them (nz <= 4) and with one (nz = 5): the tile shapes agree bit for bit,
    the fused step is within 1e-5 of the per-routine binary32 sweeps, and
    the plain form agrees with the oracle."""
    import oracle_lib as O
    s = synth.make_scenario("small", seed=11, nz=nz, nx=40, ny=34, wetdep=True, run_h=0.5)
    s.met["prate"][:] = np.float32(2.0 / 3600.0)
    res = []
    for tile in (0, 3):
        g, log = _run(s, F.PREC_FP32, 1, tile, max_steps=10)
        res.append((g.fields(), log, g.outputs()))
    for k in ("c", "cdry", "cwet"):
        assert_same_bits(res[1][0][k], res[0][0][k], k)
    gu, lu = _run(s, F.PREC_FP32, 0, max_steps=10)
    ou = gu.outputs()
    assert np.array_equal(res[1][1]["iiter"], lu["iiter"])
    for k in ("load", "col_mass", "c_grnd"):
        assert _rel(res[1][2][k], ou[k]) <= 1e-5, k
    assert np.max(res[1][2]["load"]) > 0.0
    g64, l64 = _run(s, F.PREC_FP64, max_steps=10)
    o = O.OracleCtx(s, nthreads=4)
    lo = o.run(max_steps=10)
    assert np.array_equal(l64["iiter"], lo["iiter"])
    c64, co = g64.fields()["c"], o.fields()["c"]
    assert np.max(np.abs(c64 - co)) <= 1e-12 * np.max(np.abs(co))
