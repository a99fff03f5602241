"""Aggregation in transport (f3d_set_aggregation: agrpar after the updates,
agrsrc every ndtagr steps in setsrc) through the CUDA context against the
oracle, whose restatement is pinned bit for bit to the reference's own
Fortran (tests/golden/small_aggregation.npz).

Plain FP64 form: the whole run agrees with the oracle to 1e-12 (c, deposits,
the budget log and the aggregate mass Maggr); the residual comes from CUDA's
pow/exp/log10 in the aggregation kernels and the settling chain.  Precision
form: every tile shape agrees bit for bit, and the column load agrees with
the FP64 form to 1e-4."""
import numpy as np
import pytest

import fall3d_gb300 as F
import oracle_lib as O
from fall3d_gb300 import synth
from helpers import assert_close, assert_same_bits

pytestmark = pytest.mark.gpu

OVER = dict(nc=7, phimin=3.0, phimax=8.0, aggregate=[0.2, 1000.0, 0.2], M0=1e7, run_h=0.75)


def _scen():
    s = synth.make_scenario("small", seed=9, **OVER)
    synth.add_gas_class(s)
    return s, synth.aggregation_inputs(s)


def test_run_fp64_with_aggregation():
    s, agg = _scen()
    o = O.OracleCtx(s, nthreads=8)
    o.set_aggregation(agg)
    lo = o.run()
    g = F.Context(s, F.PREC_FP64)
    g.set_aggregation(agg)
    lg = g.run()
    assert g.state()["iiter"] == o.state()["iiter"]
    assert np.array_equal(lg["iiter"], lo["iiter"])
    for k in ("time", "dt"):
        assert_close(lg[k], lo[k], 1e-14, 0.0, k)
    for k in ("massvol", "massdep", "outmass"):
        assert_close(lg[k], lo[k], 1e-12, 0.0, k)
    fo, fg = o.fields(), g.fields()
    for k in ("c", "cdry", "cwet"):
        assert_close(fg[k], fo[k], 1e-12, 1e-9, k)
    mo, mg = o.maggr(), g.maggr()
    assert np.count_nonzero(mo) > 100
    assert_close(mg, mo, 1e-12, 1e-9, "maggr")
    # the aggregate class gains what the others lose: the run differs from
    # one without aggregation
    g0 = F.Context(s, F.PREC_FP64)
    g0.run()
    assert not np.array_equal(g0.fields()["c"][s.grid["np"] - 1], fg["c"][s.grid["np"] - 1])


def test_fp32_with_aggregation():
    s, agg = _scen()
    res = {}
    for name, prec, fused, tile in (("t0", F.PREC_FP32, 1, 0), ("t3", F.PREC_FP32, 1, 3),
                                    ("fp64", F.PREC_FP64, 0, 0)):
        g = F.Context(s, prec)
        if prec == F.PREC_FP32:
            g.set_option(F.OPT_FUSED, fused)
            g.set_option(F.OPT_TILE, tile)
        g.set_aggregation(agg)
        log = g.run()
        res[name] = (g.fields(), log, g.outputs(), g.maggr())
    for k in ("c", "cdry", "cwet"):
        assert_same_bits(res["t3"][0][k], res["t0"][0][k], k)
    assert_same_bits(res["t3"][3], res["t0"][3], "maggr")
    assert np.array_equal(res["t3"][1]["iiter"], res["fp64"][1]["iiter"])
    for k in ("load", "col_mass"):
        ref = res["fp64"][2][k]
        assert np.max(np.abs(res["t3"][2][k] - ref)) <= 1e-4 * np.max(np.abs(ref)), k
    ref = res["fp64"][3]
    assert np.max(np.abs(res["t3"][3] - ref)) <= 1e-4 * np.max(np.abs(ref))


def test_aggregation_rejected_without_aggregate_class_and_in_batch():
    s = synth.make_scenario("small", seed=9, nc=5)
    g = F.Context(s, F.PREC_FP32)
    with pytest.raises(F.F3DError):
        g.set_aggregation(dict(Df=3.0, ndtagr=1, fc=np.full(5, 0.2)))
    s2, agg = _scen()
    g2 = F.Context(s2, F.PREC_FP32)
    g2.set_aggregation(agg)
    b = F.Batch(2)
    with pytest.raises(F.F3DError):
        b.add(g2)
    b.close()


def test_maggr_output():
    s, agg = _scen()
    g = F.Context(s, F.PREC_FP64)
    g.set_aggregation(agg)
    g.run(max_steps=8)
    m = g.maggr()
    assert_same_bits(g.output(F.OUT_MAGGR), m, "maggr")
    lib = O.load()
    nz, ny, nx = m.shape
    asl = np.ascontiguousarray(m.copy())
    lib.orc_ter2asl(O.p(asl), O.p(np.ascontiguousarray(s.grid["topg"], dtype=np.float64)),
                    O.p(np.ascontiguousarray(s.grid["zlayer"], dtype=np.float64)), nx, ny, nz)
    assert_same_bits(g.output(F.OUT_MAGGR, asl=True), asl, "maggr asl")
