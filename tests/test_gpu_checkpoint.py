"""Checkpoint / restart (f3d_ctx_save / f3d_ctx_restore): a run saved in
the middle of a meteo interval and restored into a fresh context continues
exactly as the uninterrupted run, bit for bit, in both forms."""
import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import synth
from helpers import assert_same_bits

pytestmark = pytest.mark.gpu


def _scen():
    # two meteo intervals (updates at 0 and 1800 s) and wet deposition
    return synth.make_scenario("small", seed=41, run_h=1.0, met_dt_h=0.5, wetdep=True)


@pytest.mark.parametrize("prec", [F.PREC_FP64, F.PREC_FP32])
@pytest.mark.parametrize("k", [7, 60])  # inside the first / the second meteo interval
def test_restart_continues_bitwise(tmp_path, prec, k):
    s = _scen()
    ref = F.Context(s, prec)
    log_ref = ref.run()
    f_ref, st_ref = ref.fields(), ref.state()
    ref.close()

    a = F.Context(s, prec)
    a.run(max_steps=k)
    path = tmp_path / "run.ckpt"
    a.save(path)
    a.close()
    b = F.Context(s, prec)
    b.restore(path)
    log_b = b.run()
    f_b, st_b = b.fields(), b.state()
    b.close()

    assert st_b["iiter"] == st_ref["iiter"] and st_b["time"] == st_ref["time"]
    assert st_b["erumass"] == st_ref["erumass"] and st_b["outmass"] == st_ref["outmass"]
    assert st_b["cd"] == st_ref["cd"]
    for key in ("c", "cdry", "cwet"):
        assert_same_bits(f_b[key], f_ref[key], key)
    # the budget records written after the restart are those of the same steps
    n = len(log_b["iiter"])
    assert n > 0
    for key in ("iiter", "massvol", "massdep", "outmass", "erumass"):
        assert np.array_equal(log_b[key], log_ref[key][-n:]), key


def test_restore_rejects_other_grid(tmp_path):
    s = _scen()
    a = F.Context(s, F.PREC_FP32)
    path = tmp_path / "run.ckpt"
    a.save(path)
    other = F.Context(synth.make_scenario("tiny", seed=1), F.PREC_FP32)
    with pytest.raises(F.F3DError):
        other.restore(path)
    with pytest.raises(F.F3DError):
        F.Context(s, F.PREC_FP64).restore(path)


@pytest.mark.parametrize("prec", [F.PREC_FP64, F.PREC_FP32])
def test_restart_with_aggregation(tmp_path, prec):
    """Aggregation in transport: the checkpoint carries Maggr, the agrsrc step
    counter and the agrpar calls since the meteo update (a source update in
    between scales vset of class iaggr once more), so a run saved after the
    source update and before the next meteo update continues bit for bit."""
    s = synth.make_scenario("small", seed=9, nc=7, phimin=3.0, phimax=8.0, aggregate=[0.2, 1000.0, 0.2],
                            M0=1e7, run_h=1.0, met_dt_h=0.5, erupt_h=0.25)
    synth.add_gas_class(s)
    agg = synth.aggregation_inputs(s)
    ref = F.Context(s, prec)
    ref.set_aggregation(agg)
    log_ref = ref.run()
    f_ref, m_ref = ref.fields(), ref.maggr()
    times = log_ref["time"]
    ref.close()
    # a step between the source update (900 s) and the next meteo update
    probe = F.Context(s, prec)
    probe.set_aggregation(agg)
    k = 0
    while True:
        k += 1
        probe.run(max_steps=1)
        if probe.state()["time"] > 1000.0:
            break
    assert probe.state()["time"] < 1800.0
    probe.close()
    a = F.Context(s, prec)
    a.set_aggregation(agg)
    a.run(max_steps=k)
    path = tmp_path / "agg.ckpt"
    a.save(path)
    a.close()
    b = F.Context(s, prec)
    b.set_aggregation(agg)
    b.restore(path)
    b.run()
    for key in ("c", "cdry", "cwet"):
        assert_same_bits(b.fields()[key], f_ref[key], key)
    assert_same_bits(b.maggr(), m_ref, "maggr")
    assert len(times) > 0
    # a context without aggregation refuses the checkpoint
    with pytest.raises(F.F3DError):
        F.Context(s, prec).restore(path)
