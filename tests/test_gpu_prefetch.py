"""The look-ahead meteo update of f3d_run (F3D_OPT_PREFETCH): the next DBS
snapshot's update (Sources/meteo.f90:27-149) is computed on a second stream
into a second set of the coefficient fields while the current interval
steps, and the sets are exchanged when the update is due.  It changes no
result: with it on and off the runs agree bit for bit in both forms over
several meteo updates (fields, deposits, budgets, the time and dt
sequences, the settling iteration counts); a run resumed in pieces and a run
restored from a checkpoint taken while a look-ahead update was in flight
continue bit for bit."""
import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import synth
from helpers import assert_same_bits

pytestmark = pytest.mark.gpu


def _scen():
    # 15-minute DBS intervals over 2 h: eight meteo updates
    return synth.make_scenario("small", seed=21, run_h=2.0, met_dt_h=0.25, wetdep=True)


def _run(s, prec, pref, **kw):
    g = F.Context(s, prec)
    g.set_option(F.OPT_PREFETCH, pref)
    assert g.get_option(F.OPT_PREFETCH) == pref
    log = g.run(**kw)
    return g, log


def _same(ga, la, gb, lb):
    for k in la:
        assert_same_bits(np.asarray(la[k], float), np.asarray(lb[k], float), "log " + k)
    fa, fb = ga.fields(), gb.fields()
    for k in ("c", "cdry", "cwet", "vset", "vdep"):
        assert_same_bits(fa[k], fb[k], k)
    assert np.array_equal(ga.iters(), gb.iters())
    oa, ob = ga.outputs(), gb.outputs()
    for k in oa:
        assert_same_bits(oa[k], ob[k], k)
    sa, sb = ga.state(), gb.state()
    assert sa == sb


@pytest.mark.parametrize("prec", [F.PREC_FP32, F.PREC_FP64])
def test_lookahead_changes_no_result(prec):
    s = _scen()
    s.met["prate"][:] = np.float32(2.0 / 3600.0)
    ga, la = _run(s, prec, 0)
    gb, lb = _run(s, prec, 1)
    assert ga.state()["time"] >= 7200.0 and len(la["iiter"]) >= 12
    _same(ga, la, gb, lb)


def test_lookahead_resume_and_checkpoint(tmp_path):
    s = _scen()
    whole, lw = _run(s, F.PREC_FP32, 1)
    # in pieces: each call stops inside an interval, with the next update looked ahead
    g = F.Context(s, F.PREC_FP32)
    g.set_option(F.OPT_PREFETCH, 1)
    for t in (1000.0, 2500.0, 4100.0):
        g.run(end_time=t)
    path = tmp_path / "mid.ckpt"
    g.save(path)  # a look-ahead update is in flight or ready
    g.run()
    assert_same_bits(g.fields()["c"], whole.fields()["c"], "resumed")
    # restored into a new context, continuing with the look-ahead on
    r = F.Context(s, F.PREC_FP32)
    r.set_option(F.OPT_PREFETCH, 1)
    r.restore(path)
    r.run()
    assert_same_bits(r.fields()["c"], whole.fields()["c"], "restored")
    assert r.state()["iiter"] == whole.state()["iiter"]
    # a direct meteo update drops the look-ahead: the run still equals one made without it
    a, la = _run(s, F.PREC_FP32, 1, end_time=1000.0)
    a.meteo(1)
    b, lb = _run(s, F.PREC_FP32, 0, end_time=1000.0)
    b.meteo(1)
    assert_same_bits(a.fields()["vset"], b.fields()["vset"], "vset after a direct update")
