"""A run restarted from the reference's restart file (fall3d_gb300/restart.py):
the plain FP64 form writes the file at the end of a first run, a new context
reads it (c and the masses from the file, cdry and cwet zero, the drag chain
at its initial value: rearst.f90 / setup.f90:116) and continues; the oracle
continues from the same file.  Tolerances of tests/test_gpu_run.py (1e-12,
bit-exact steps)."""
import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import restart, synth
import oracle_lib as O
from helpers import compare_runs

pytestmark = pytest.mark.gpu


def test_continue_from_reference_restart(tmp_path):
    pytest.importorskip("scipy")
    s = synth.make_scenario("small", seed=31, run_h=1.0)
    bounds = (0.0, 1.0, 0.0, 1.0)
    first = F.Context(s, F.PREC_FP64)
    first.run(end_time=1800.0)
    path = tmp_path / "small.rst.nc"
    restart.save_reference_restart(first, path, 0.0, 1800.0, bounds)
    # the continuation: a new run from 1800 s with the restart's state
    g = F.Context(s, F.PREC_FP64)
    r = restart.load_reference_restart(g, path, bounds)
    lg = g.run(beg_time=1800.0)
    o = O.OracleCtx(s, nthreads=8)
    z = np.zeros((s.grid["nc"] + 1, s.grid["ny"], s.grid["nx"]))
    o.upload_state(np.ascontiguousarray(r["c"]), z, z, r["erumass"], r["outmass"], 1.0)
    lo = o.run(beg_time=1800.0)
    compare_runs(o, lo, g, lg)
    assert np.max(np.abs(r["c"] - first.fields()["c"])) <= 1e-6 * np.max(np.abs(first.fields()["c"]))
