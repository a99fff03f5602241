"""Whole-run parity: the Fall3d.f90 time loop through the CUDA context
(f3d_run) against the same loop in the CPU oracle (orc_run).

Plain FP64 form: bit-exact integer bookkeeping (step count, source-cell
indices) and 1e-12 relative agreement in concentration, ground deposit,
column load and the mass budget.  The transport arithmetic itself is
bit-identical; the residual differences come from CUDA's pow/log10 in the
coefficient chain (a few ulp in vset, rkhor) carried through the steps.
Per-cell concentrations are compared with a floor of 1e-9 x max|c| below
which a cell counts as empty: cells that small are the result of
cancellation at the plume edge, where a relative measure carries no
information.
"""
import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import synth
import oracle_lib as O
from helpers import assert_same_bits, compare_runs

pytestmark = pytest.mark.gpu

RTOL = 1e-12
FLOOR = 1e-9


def _run_both(scen, precision=F.PREC_FP64, max_steps=0):
    o = O.OracleCtx(scen, nthreads=8)
    lo = o.run(max_steps=max_steps)
    g = F.Context(scen, precision)
    lg = g.run(max_steps=max_steps)
    return o, lo, g, lg


_compare = compare_runs


def test_tiny_run_fp64():
    s = synth.make_scenario("tiny", seed=1)
    o, lo, g, lg = _run_both(s)
    _compare(o, lo, g, lg)


def test_small_run_fp64_wet_deposition():
    s = synth.make_scenario("small", seed=2, wetdep=True, run_h=1.0)
    s.met["prate"][:] = np.float32(2.0 / 3600.0)  # 2 mm/h everywhere, as mm/s
    o, lo, g, lg = _run_both(s)
    fo, fg = _compare(o, lo, g, lg)
    assert fo["cwet"].max() > 0


def test_cfg0_full_run_fp64():
    """The CPU-sized workload: 80x80x25, 6 classes, 3 h."""
    s = synth.make_scenario("cfg0", seed=0)
    o, lo, g, lg = _run_both(s)
    _compare(o, lo, g, lg)
    # the vsettl iteration counts of the last meteo update agree exactly
    assert np.array_equal(g.iters(), o.iters())


def test_fp32_form_vs_fp64_form():
    """Precision form: identical step sequence (finddt in binary64), column
    load and ground deposit within 1e-4 of the FP64 form."""
    s = synth.make_scenario("small", seed=4, run_h=1.5)
    g64 = F.Context(s, F.PREC_FP64)
    l64 = g64.run()
    g32 = F.Context(s, F.PREC_FP32)
    l32 = g32.run()
    assert np.array_equal(l32["iiter"], l64["iiter"])
    assert_same_bits(l32["dt"], l64["dt"], "dt sequence")
    assert_same_bits(l32["time"], l64["time"], "time sequence")
    o64, o32 = g64.outputs(), g32.outputs()
    for k in ("load", "col_mass"):
        e = np.max(np.abs(o32[k] - o64[k])) / np.max(np.abs(o64[k]))
        assert e <= 1e-4, (k, e)
    tot64 = l64["massvol"] + l64["massdep"] + l64["outmass"]
    tot32 = l32["massvol"] + l32["massdep"] + l32["outmass"]
    assert np.max(np.abs(tot32 - tot64) / tot64) <= 1e-5


def test_run_in_pieces_equals_one_run():
    """f3d_run resumes where it stopped (the loop state lives in the context)."""
    s = synth.make_scenario("tiny", seed=3)
    a = F.Context(s)
    a.run()
    b = F.Context(s)
    b.run(max_steps=7)
    b.run(max_steps=5)
    b.run()
    assert a.state()["iiter"] == b.state()["iiter"]
    assert_same_bits(b.fields()["c"], a.fields()["c"], "resumed run")


def test_step_api_matches_run_and_is_deterministic():
    s = synth.make_scenario("tiny", seed=5)
    r = F.Context(s)
    r.run(max_steps=10)
    x = F.Context(s)
    x.source(0)
    x.meteo(0)
    for _ in range(10):
        x.step()
    assert x.state()["iiter"] == 10
    assert_same_bits(x.fields()["c"], r.fields()["c"], "step API vs run")


def test_errors_are_status_codes():
    s = synth.make_scenario("tiny", seed=1)
    g = F.Context(s)
    with pytest.raises(F.F3DError) as e:
        g.step()  # before any meteo
    assert e.value.code == 4
    bad = dict(s.grid)
    bad["nx"] = 2
    with pytest.raises(F.F3DError):
        F.Context(synth.Scenario("bad", 0, bad, s.met, s.src, 0.0, 1.0))


def test_run_in_pieces_equals_one_run():
    """f3d_run called with increasing end times continues the one run: the
    meteo and source updates that the end of a call switched off are due again
    in the next call (the DBS updates at 1800 s and 3600 s fall in the second
    and third pieces), bit for bit in the FP32 form and to the oracle's
    tolerance in the FP64 form."""
    s = synth.make_scenario("small", seed=41, run_h=1.5, met_dt_h=0.5)
    for prec in (F.PREC_FP32, F.PREC_FP64):
        whole = F.Context(s, prec)
        lw = whole.run()
        part = F.Context(s, prec)
        for t in (1000.0, 2500.0, 4000.0, s.end_time):
            part.run(end_time=t)
        assert part.state()["iiter"] == whole.state()["iiter"]
        assert np.array_equal(part.fields()["c"], whole.fields()["c"])
        assert np.array_equal(part.fields()["vset"], whole.fields()["vset"])
    o = O.OracleCtx(s, nthreads=8)
    for t in (1000.0, 2500.0, 4000.0, s.end_time):
        o.run(end_time=t)
    assert o.state()["iiter"] == whole.state()["iiter"]
    assert lw["iiter"][-1] == o.state()["iiter"]
