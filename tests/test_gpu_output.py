"""Output variables of Sources/printres_nc.f90 computed on the device
(f3d_output, f3d_output_fl) against the oracle's restatement on the same
state: every variable, in both forms, agrees bit for bit (binary64 in the
reference's order of operations on the downloaded state), and the binary32
results are the binary64 ones rounded once."""
import numpy as np
import pytest

import fall3d_gb300 as F
import oracle_lib as O
from fall3d_gb300 import synth

pytestmark = pytest.mark.gpu

# fine classes (diameters 125, 54, 24, 10.3, 4.5 and 1.95 um) so that the
# PM05/PM10/PM20 and aerosol selections are not empty; the last class is a
# gas (np = nc - 1)
OVER = dict(nx=30, ny=26, nz=14, nc=6, phimin=3.0, phimax=9.0, wetdep=True, run_h=0.6, M0=3e6)

VARS = [(F.OUT_LOAD, i) for i in range(0, 6)] + [(F.OUT_WET, i) for i in range(0, 6)] + [
    (F.OUT_THICK, 0), (F.OUT_COL_MASS, 0), (F.OUT_COL_MASS, 1), (F.OUT_PM_COL, 5), (F.OUT_PM_COL, 10),
    (F.OUT_PM_COL, 20), (F.OUT_C_GRND, 0), (F.OUT_PM_GRND, 5), (F.OUT_PM_GRND, 10), (F.OUT_PM_GRND, 20),
    (F.OUT_AOT05, 0)] + [(F.OUT_CON, i) for i in range(0, 7)]


def _scenario():
    s = synth.make_scenario("small", seed=31, **OVER)
    s.grid["np"] = s.grid["nc"] - 1
    return s


@pytest.fixture(scope="module", params=[F.PREC_FP64, F.PREC_FP32])
def run(request):
    s = _scenario()
    g = F.Context(s, request.param)
    g.run()
    yield s, g, g.fields()
    g.close()


@pytest.mark.parametrize("var,index", VARS)
def test_output_matches_oracle(run, var, index):
    s, g, f = run
    for asl in ((False, True) if var == F.OUT_CON else (False,)):
        got = g.output(var, index, asl=asl)
        want = O.output(s.grid, f, var, index, asl=asl)
        assert got.shape == want.shape
        assert np.array_equal(got, want), (var, index, asl, np.max(np.abs(got - want)))
        g32 = g.output(var, index, asl=asl, binary32=True)
        assert g32.dtype == np.float32 and np.array_equal(g32, got.astype(np.float32))


def test_selections_not_empty(run):
    s, g, f = run
    assert np.max(g.output(F.OUT_PM_COL, 5)) > 0.0
    assert np.max(g.output(F.OUT_AOT05)) > 0.0
    assert np.max(g.output(F.OUT_COL_MASS, 1)) > 0.0  # the gas class
    assert np.max(g.output(F.OUT_WET)) > 0.0


@pytest.mark.parametrize("fl", [0.0, 50.0, 100.0, 180.0, 300.0, 400.0])
def test_flight_level_matches_oracle(run, fl):
    s, g, f = run
    gr = s.grid
    zabs = gr["zlayer"][:, None, None] + gr["topg"][None]
    pres = synth.standard_atmosphere(zabs)[1]
    got = g.output_fl(fl, pres)
    want = O.output(gr, f, "fl", p_levels=pres, flight_level=fl)
    assert np.array_equal(got, want), (fl, np.max(np.abs(got - want)))
    assert np.array_equal(g.output_fl(fl, pres, binary32=True), got.astype(np.float32))


def test_outputs_triplet_is_the_same_variables(run):
    s, g, f = run
    o = g.outputs()
    assert np.array_equal(o["load"], g.output(F.OUT_LOAD, 0))
    assert np.array_equal(o["col_mass"], g.output(F.OUT_COL_MASS, 0))
    assert np.array_equal(o["c_grnd"], g.output(F.OUT_C_GRND, 0))


def test_output_rejects_bad_selectors(run):
    s, g, f = run
    for var, index in ((F.OUT_LOAD, 6), (F.OUT_COL_MASS, 2), (F.OUT_PM_COL, 7), (F.OUT_CON, 7), (99, 0)):
        with pytest.raises(F.F3DError):
            g.output(var, index)


def test_track_points_match_oracle(run):
    """Tracking points (writps, writps_air, writps_end) at points inside
    the grid, on a node and in the last cell: bitwise equal to the
    oracle's restatement on the same state."""
    s, g, f = run
    gr = s.grid
    xo, yo = s.info["origin"]
    nx, ny = gr["nx"], gr["ny"]
    xs = np.array([xo + 0.37 * gr["dx"] * (nx - 1), xo + 3 * gr["dx"], xo + (nx - 1.5) * gr["dx"]])
    ys = np.array([yo + 0.61 * gr["dy"] * (ny - 1), yo + 5 * gr["dy"], yo + 0.5 * gr["dy"]])
    got = g.track_points(xs, ys, xo, yo)
    want = O.track_points(gr, f, xs, ys, xo, yo)
    assert got.shape == want.shape
    assert np.array_equal(got, want), np.max(np.abs(got - want))
    assert np.max(got[:, 0]) > 0.0
    with pytest.raises(F.F3DError):
        g.track_points(np.array([xo - 1.0]), np.array([yo]), xo, yo)
