"""A run whose meteorology comes from a DBS file: the met of a synthetic
scenario is written on its own set of levels (SetDbs schema), read back on
the model levels through fall3d_gb300.dbs.read_dbs (get_dbs_value_plane's
interval selection and vertical interpolation, reamet's defaults), and the
plain FP64 form runs f3d_run on it; the oracle runs the same series.
Tolerances as in tests/test_gpu_run.py (1e-12 relative, bit-exact steps)."""
import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import dbs, synth
import oracle_lib as O
from helpers import compare_runs

pytestmark = pytest.mark.gpu


def test_run_from_dbs_file(tmp_path):
    pytest.importorskip("scipy")
    s = synth.make_scenario("small", seed=12, wetdep=True, run_h=1.0, max_snapshots=3)
    s.met["prate"][:] = np.float32(1.5 / 3600.0)
    zl = np.asarray(s.grid["zlayer"])
    # the database's own levels: every other model level and one above the top
    alt = np.concatenate([zl[::2], [zl[-1] + 500.0]]).astype(np.float32)
    idx = np.minimum(np.searchsorted(zl, alt), len(zl) - 1)
    met = {k: np.asarray(s.met[k])[:, idx] for k in ("u", "v", "w", "t", "tp", "rho")}
    met.update({k: s.met[k] for k in ("ust", "pblh", "rmol", "znt", "prate", "ldu", "times")})
    path = tmp_path / "small.nc"
    dbs.write_dbs(path, met, alt)
    series, warnings = dbs.read_dbs(path, zl, wetdep=True)
    assert not warnings
    s.met = series
    o = O.OracleCtx(s, nthreads=8)
    lo = o.run()
    g = F.Context(s, F.PREC_FP64)
    lg = g.run()
    compare_runs(o, lo, g, lg)
    assert len(lg["iiter"]) > 2 and g.state()["time"] >= 3600.0  # a meteo update from the second record
