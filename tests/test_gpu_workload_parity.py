"""Plain FP64 form against the oracle on the benchmarked workload and on a
slice of the large stress workload, through the C ABI (f3d_run).

The benchmarked workload is 400x300x50 at 0.02 deg with 16 classes
(phi -2..6), a k^-5/3 wind perturbation, two base states interpolated in
time, a precipitation band (wet deposition on) and a 15 km Suzuki column:
the scenario bench.py times, built by the same call.  The run starts 60 s
before the first DBS boundary, so it performs the first meteo update, about
ten steps, the second meteo update (the drag-coefficient chain of setvset
continues from the first one, setvset.f90:89) and ten more steps.

The stress slice keeps the large workload's class set (30 classes, the last
one an aggregate class with 20% of the fine ash), 80 levels up to 30 km,
0.01 deg spacing, wet deposition and a 25 km column, on a 120x100 sub-domain
the oracle finishes in seconds.

Tolerances as in tests/test_gpu_run.py: 1e-12 relative (cells below 1e-9 x
max count as empty) for c, cdry, cwet, LOAD, COL_MASS, C_GRND and the
budgets; bit-exact step counts and settling iteration counts; time and dt
sequences to 1e-14.
"""
import os

import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import synth
import oracle_lib as O
from helpers import assert_close, compare_runs

pytestmark = pytest.mark.gpu

NTHREADS = max(1, min(16, os.cpu_count() or 1))


def _run_both(s, beg_time, max_steps):
    o = O.OracleCtx(s, nthreads=NTHREADS)
    lo = o.run(beg_time=beg_time, max_steps=max_steps)
    g = F.Context(s, F.PREC_FP64)
    lg = g.run(beg_time=beg_time, max_steps=max_steps)
    return o, lo, g, lg


def test_benchmarked_workload_fp64_across_a_meteo_update():
    s = synth.make_scenario("cfg1", seed=0, max_snapshots=3)
    t_dbs = float(s.met["times"][1])
    o, lo, g, lg = _run_both(s, t_dbs - 60.0, 20)
    fo, fg = compare_runs(o, lo, g, lg)
    st = g.state()
    assert st["time"] > t_dbs  # the second meteo update happened
    assert len(lg["iiter"]) >= 2  # budget records before and after it
    # the settling iteration counts of the second update agree exactly
    assert np.array_equal(g.iters(), o.iters())
    # the features of the workload were exercised: wet deposit, dry deposit
    # and mass in every class
    assert fo["cwet"][1:].max() > 0.0
    assert fo["cdry"][1:].max() > 0.0
    assert all(fo["c"][ic].max() > 0.0 for ic in range(s.grid["nc"]))


def test_stress_class_set_fp64_slice():
    s = synth.make_scenario("cfg4", seed=0, nx=120, ny=100, max_snapshots=2)
    assert s.grid["nc"] == 30 and s.info["classes"][-1].lower().startswith("agg")
    o, lo, g, lg = _run_both(s, None, 12)
    compare_runs(o, lo, g, lg)
    assert np.array_equal(g.iters(), o.iters())


def test_reference_size_full_run_against_the_reference():
    """The CPU-runnable workload (80x80x25 at 0.05 deg, 6 classes, 3 h: 550
    steps, three meteo updates, the eruption's end) run in full by the plain
    FP64 form and compared with the reference's own run of it
    (tests/golden/cfg0_full_run.npz, the translated Fortran): bit-exact step
    count, time and dt sequences to 1e-14, the mass-budget log and every
    sampled concentration, ground deposit and the outputs to 1e-12.  The
    precision form takes the same steps, and its LOAD and COL_MASS are within
    1e-4 of the FP64 form's."""
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    gold = np.load(os.path.join(here, "cfg0_full_run.npz"))
    stride = int(gold["sample_stride"])
    s = synth.make_scenario("cfg0", seed=0)
    g = F.Context(s, F.PREC_FP64)
    lg = g.run()
    st = g.state()
    assert st["iiter"] == int(gold["iiter"]) == 550
    assert np.array_equal(lg["iiter"], gold["log_iiter"].astype(lg["iiter"].dtype))
    for k in ("time", "dt", "dtc", "erumass"):
        assert_close(lg[k], gold["log_" + k], 1e-14, 0.0, k)
    for k in ("massvol", "massdep", "massdry", "masswet", "outmass"):
        assert_close(lg[k], gold["log_" + k], 1e-12, 0.0, k)
    f = g.fields()
    assert_close(f["c"].ravel()[::stride], gold["c"].ravel(), 1e-12, 1e-9, "c")
    assert_close(f["cdry"], gold["cdry"], 1e-12, 1e-9, "cdry")
    assert_close(f["cwet"], gold["cwet"], 1e-12, 1e-9, "cwet")
    assert_close(np.array([st["outmass"]]), np.array([float(gold["outmass"])]), 1e-12, 0.0, "outmass")
    # the reference scheme's own budget closure over the run, reproduced
    eru = lg["erumass"][-1]
    closure = (lg["massvol"][-1] + lg["massdep"][-1] + lg["outmass"][-1] - eru) / eru
    gclosure = (gold["log_massvol"][-1] + gold["log_massdep"][-1] + gold["log_outmass"][-1] - eru) / eru
    assert abs(closure - gclosure) <= 1e-10
    out64 = g.outputs()
    g32 = F.Context(s, F.PREC_FP32)
    l32 = g32.run()
    assert g32.state()["iiter"] == 550 and np.array_equal(l32["dt"], lg["dt"])
    out32 = g32.outputs()
    for k in ("load", "col_mass"):
        assert_close(out32[k], out64[k], 1e-4, 1e-9, k)
