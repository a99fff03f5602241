"""Shared helpers for the parity tests (test infrastructure)."""
from __future__ import annotations

import numpy as np

from fall3d_gb300 import synth
import oracle_lib


def assert_same_bits(a, b, what=""):
    """Bitwise equality, except that NaN payloads/signs are not compared
    (x86 and CUDA produce default NaNs of opposite sign)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    na, nb = np.isnan(a), np.isnan(b)
    assert np.array_equal(na, nb), f"{what}: NaN positions differ ({na.sum()} vs {nb.sum()})"
    ua = a[~na].view(np.uint64)
    ub = b[~nb].view(np.uint64)
    bad = np.nonzero(ua != ub)[0]
    if len(bad):
        i = bad[0]
        raise AssertionError(f"{what}: {len(bad)} of {ua.size} values differ bitwise; first "
                             f"{a[~na][i]!r} vs {b[~nb][i]!r}")


def rel_err(a, b, floor_frac=0.0):
    """max |a-b| / max(|b|, floor) with floor = floor_frac * max|b|."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.max(np.abs(b)) if b.size else 0.0
    den = np.maximum(np.abs(b), floor_frac * scale)
    den[den == 0] = 1.0
    return float(np.max(np.abs(a - b) / den)) if a.size else 0.0


def assert_close(a, b, rtol, floor_frac, what=""):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert np.array_equal(np.isnan(a), np.isnan(b)), f"{what}: NaN positions differ"
    m = ~np.isnan(b)
    e = rel_err(a[m], b[m], floor_frac)
    assert e <= rtol, f"{what}: relative error {e:.3e} > {rtol:.1e}"
    return e


def oracle_state(name="tiny", seed=1, steps=5, **over):
    """Scenario + oracle context after one meteo update, one source and
    ``steps`` steps: a plume-bearing state for the per-routine tests."""
    s = synth.make_scenario(name, seed=seed, **over)
    o = oracle_lib.OracleCtx(s)
    o.source(0)
    o.meteo(0)
    for _ in range(steps):
        o.step()
    return s, o


def compare_runs(o, lo, g, lg, rtol=1e-12, floor=1e-9):
    """The FP64 context against the oracle after the same run: bit-exact
    step counts, the time/dt sequence to 1e-14, and ``rtol`` (cells below
    ``floor`` x max count as empty) in the budgets, the fields and the
    outputs LOAD / COL_MASS / C_GRND.  Returns both field sets."""
    so, sg = o.state(), g.state()
    assert sg["iiter"] == so["iiter"]
    assert np.array_equal(lg["iiter"], lo["iiter"])
    for k in ("time", "dt", "dtc", "erumass"):
        assert_close(lg[k], lo[k], 1e-14, 0.0, k)
    for k in ("massvol", "massdep", "massdry", "outmass"):
        assert_close(lg[k], lo[k], rtol, 0.0, k)
    fo, fg = o.fields(), g.fields()
    assert_close(fg["c"], fo["c"], rtol, floor, "c")
    assert_close(fg["cdry"], fo["cdry"], rtol, floor, "cdry")
    assert_close(fg["cwet"], fo["cwet"], rtol, floor, "cwet")
    oo, og = o.outputs(), g.outputs()
    for k in ("load", "col_mass", "c_grnd"):
        assert_close(og[k], oo[k], rtol, floor, k)
    return fo, fg
