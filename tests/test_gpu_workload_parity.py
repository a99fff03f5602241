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
from helpers import compare_runs

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
