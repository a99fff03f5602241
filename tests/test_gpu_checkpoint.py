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
