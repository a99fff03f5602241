"""The driver of the translated reference (oracle/ref_driver.py), which
bench.py times as the reference's CPU path: its class groups follow
Sources/Parallel.F90 localdim/globalindex, and stepping the classes in
groups (the reference's class decomposition, one process per group in the
timing) gives every class the concentrations of the serial run bit for bit,
so the timed parallel run does the serial run's work."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import ref_driver  # noqa: E402
from fall3d_gb300 import synth  # noqa: E402


def _have_reference():
    import ref_translate

    try:
        ref_translate.build()
        return True
    except Exception:
        return False


def test_class_groups_follow_localdim_and_globalindex():
    for nc in (1, 5, 6, 16, 30):
        for ngrp in range(1, nc + 1):
            g = ref_driver.class_groups(nc, ngrp)
            assert len(g) == ngrp
            assert sum(n for _, n in g) == nc
            assert g[0][0] == 1
            for (a, n), (b, _) in zip(g, g[1:]):
                assert b == a + n
            sizes = [n for _, n in g]
            assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)


@pytest.mark.skipif(not _have_reference(), reason="translated reference unavailable")
def test_class_groups_step_the_serial_run():
    s = synth.make_scenario("tiny", seed=3, max_snapshots=2)
    nc = s.grid["nc"]
    steps = 6

    def run(ic_loc, nc_loc):
        r = ref_driver.RefRun(s, ic_loc=ic_loc, nc_loc=nc_loc)
        r.source(0)
        r.meteo(0)
        for _ in range(steps):
            r.step()
        nx, ny, nz, _ = r.dims
        h = (nx + 2) * (ny + 2) * (nz + 2)
        return r.R.arr("c", h * nc).copy().reshape(nc, -1)

    serial = run(1, nc)
    assert np.any(serial > 0)
    for ic_loc, nc_loc in ref_driver.class_groups(nc, 3):
        part = run(ic_loc, nc_loc)
        sl = slice(ic_loc - 1, ic_loc - 1 + nc_loc)
        assert np.array_equal(part[sl].view(np.uint64), serial[sl].view(np.uint64)), (ic_loc, nc_loc)


@pytest.mark.skipif(not _have_reference(), reason="translated reference unavailable")
def test_class_parallel_timing_runs_every_group():
    """The forked class groups of bench.py's reference arm: every group runs
    the same number of timed steps and reports back; the work is the
    serial run's (all classes, every step)."""
    s = synth.make_scenario("tiny", seed=3, max_snapshots=2)
    nc = s.grid["nc"]
    r = ref_driver.time_class_parallel(s, 3, steps=4, serial_steps=1, budget_s=5.0)
    par, ser = r["parallel"], r["serial"]
    assert par["groups"] == 3 and 2 <= par["steps"] <= 4
    cells = s.grid["nx"] * s.grid["ny"] * s.grid["nz"]
    assert par["cell_class_steps"] == cells * nc * par["steps"]
    assert ser["cell_class_steps"] == cells * nc
    assert par["seconds"] > 0.0 and par["slowest_group_s"] <= par["seconds"] and r["meteo_s"] > 0.0
