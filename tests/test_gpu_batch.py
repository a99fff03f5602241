"""The batched precision form (f3d_batch_*): scenarios of different sizes,
class counts, time steps and lengths advanced together give, each, exactly
the result of running that scenario alone through f3d_run (same kernels,
same formulas: the concentrations agree bit for bit; the outflow budget is
summed over a different block partition, exact in double-double before the
final rounding)."""
import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import synth

pytestmark = pytest.mark.gpu

RTOL_BUDGET = 1e-14  # outmass: same terms, different reduction partition


def _members():
    return [
        synth.make_scenario("small", seed=21, run_h=0.5),
        synth.make_scenario("small", seed=22, nx=40, ny=24, nz=12, nc=5, run_h=0.75, wetdep=True,
                            M0=3e6),
        synth.make_scenario("tiny", seed=23, nx=21, ny=26, nz=10, nc=3, run_h=0.4),  # an odd nx
        synth.make_scenario("small", seed=24, nx=36, ny=36, nz=16, nc=6, run_h=0.3, H=6000.0),
    ]


def _alone(s):
    g = F.Context(s, F.PREC_FP32)
    log = g.run()
    return g.fields(), log, g.state()


@pytest.fixture(scope="module")
def alone():
    return [_alone(s) for s in _members()]


def _check_same(ref, ctx, log, tag):
    f_ref, log_ref, st_ref = ref
    st = ctx.state()
    assert st["iiter"] == st_ref["iiter"], tag
    assert st["time"] == st_ref["time"], tag
    f = ctx.fields()
    for k in ("c", "cdry", "cwet"):
        assert np.array_equal(f[k], f_ref[k], equal_nan=True), (tag, k)
    assert len(log["iiter"]) == len(log_ref["iiter"]), tag
    assert np.array_equal(log["iiter"], log_ref["iiter"]), tag
    for k in ("massvol", "massdep", "massdry", "masswet", "erumass"):
        assert np.array_equal(log[k], log_ref[k]), (tag, k)
    scale = max(1.0, float(np.max(np.abs(log_ref["outmass"]))))
    assert np.max(np.abs(log["outmass"] - log_ref["outmass"])) <= RTOL_BUDGET * scale, tag


@pytest.mark.parametrize("graph,tile", [(1, 3), (0, 3), (1, 0)])
def test_batch_equals_alone(alone, graph, tile):
    members = _members()
    b = F.Batch(8)
    b.set_option(F.OPT_GRAPH, graph)
    b.set_option(F.OPT_TILE, tile)
    ctxs, slots = [], []
    for s in members:
        g = F.Context(s, F.PREC_FP32)
        ctxs.append(g)
        slots.append(b.add(g))
    b.run()
    for i, (g, sl) in enumerate(zip(ctxs, slots)):
        st, steps, _ = b.poll(sl)
        assert st == F.Batch.DONE
        _check_same(alone[i], g, b.log(sl), f"member {i}")
    bs, ccs, n = b.stats()
    assert n == 0 and bs == max(a[2]["iiter"] for a in alone)
    b.close()


def test_batch_autotune_and_late_join(alone):
    """A member joins after the others have run for a while, and the tile
    shape is re-tuned mid-run: neither changes any result."""
    members = _members()
    b = F.Batch(8)
    ctxs = [F.Context(s, F.PREC_FP32) for s in members]
    slots = {0: b.add(ctxs[0]), 1: b.add(ctxs[1])}
    for _ in range(5):
        b.step()
    best, ms = b.autotune(reps=2)
    assert best in (0, 1, 2, 3) and min(v for v in ms if v > 0) > 0
    slots[2] = b.add(ctxs[2])
    for _ in range(3):
        b.step()
    b.set_option(F.OPT_TILE, 1)
    slots[3] = b.add(ctxs[3])
    b.run()
    for i in range(4):
        _check_same(alone[i], ctxs[i], b.log(slots[i]), f"member {i}")
    b.close()


def test_batch_rejects_plain_form():
    s = synth.make_scenario("tiny", seed=1)
    g = F.Context(s, F.PREC_FP64)
    b = F.Batch(2)
    with pytest.raises(F.F3DError):
        b.add(g)
    b.close()
