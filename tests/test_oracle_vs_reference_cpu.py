"""The CPU oracle against the reference's own Fortran (translated to C by
oracle/ref_translate.py, driven by oracle/ref_driver.py) on seeded random
small scenarios, live: every settling model, every vertical and horizontal
diffusivity model, both coordinate systems, wet deposition on and off,
stable and unstable surface layers, odd and even grid sizes, and meteo
updates inside the run (the SAVEd drag coefficient carried across them).
Agreement is bit for bit, as for the committed golden cases; this widens
the pinned option space.  Needs the reference sources (skipped without)."""
import os
import sys

import numpy as np
import pytest

import oracle_lib as O
from fall3d_gb300 import synth
from helpers import assert_same_bits

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def _have_reference():
    import ref_translate

    try:
        ref_translate.build()
        return True
    except Exception:
        return False


def _case(seed):
    r = np.random.default_rng(500 + seed)
    lonlat = bool(r.integers(0, 2))
    over = dict(nx=int(r.integers(7, 18)), ny=int(r.integers(7, 18)), nz=int(r.integers(5, 11)),
                nc=int(r.integers(2, 6)), modv=int(r.integers(1, 5)), modkv=int(r.integers(0, 3)),
                modkh=int(r.integers(0, 3)), coord=0 if lonlat else 1,
                spacing=0.05 if lonlat else 4000.0, wetdep=bool(r.integers(0, 2)),
                rmol=float(r.choice([1.0 / 500.0, -1.0 / 300.0])), met_dt_h=0.25, run_h=1.0,
                rkv0=float(r.uniform(10.0, 60.0)), rkh0=float(r.uniform(200.0, 2000.0)))
    s = synth.make_scenario("tiny", seed=seed, **over)
    if s.grid["wetdep"]:
        band = np.linspace(0.0, 4.0, s.grid["nx"])[None, :] / 3600.0
        s.met["prate"][:] = np.asarray(band, np.float32).astype(np.float64)
    return s, over


@pytest.mark.skipif(not _have_reference(), reason="translated reference unavailable")
@pytest.mark.parametrize("seed", range(12))
def test_oracle_equals_reference_on_random_options(seed):
    import ref_driver

    s, over = _case(seed)
    steps = 40
    ref = ref_driver.run(s, max_steps=steps)
    o = O.OracleCtx(s, nthreads=2)
    log = o.run(max_steps=steps)
    st = o.state()
    tag = f"seed {seed} {over}"
    assert st["iiter"] == int(ref["iiter"]), tag
    f = o.fields()
    for k in ("c", "cdry", "cwet"):
        assert_same_bits(f[k].ravel(), np.asarray(ref[k]).ravel(), f"{k} ({tag})")
    for k in ("time", "dt", "erumass", "outmass"):
        assert_same_bits(np.array([st[k]]), np.array([float(ref[k])]), f"{k} ({tag})")
    for k in ("iiter", "dt", "massvol", "massdep", "outmass"):
        assert_same_bits(np.asarray(log[k], float), np.asarray(ref["log_" + k], float), f"log {k} ({tag})")
