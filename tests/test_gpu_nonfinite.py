"""f3d_count_nonfinite: the NaN and infinite values of the concentrations
(the whole halo array of every class) and of the deposits, counted on the
device in both forms.  The values are planted through f3d_upload_state;
nothing is stepped with them."""
import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [F.PREC_FP64, F.PREC_FP32])
def test_count_nonfinite(prec):
    s = synth.make_scenario("tiny", seed=1)
    g = F.Context(s, prec)
    g.source(0)
    g.meteo(0)
    g.step(3)
    assert g.count_nonfinite() == (0, 0)
    f = g.fields()
    st = g.state()
    c, cdry, cwet = f["c"].copy(), f["cdry"].copy(), f["cwet"].copy()
    c[0, 1, 1, 1] = np.nan
    c[0, 2, 2, 2] = -np.inf
    c[-1, -1, -1, -1] = np.inf  # the last halo corner of the last class
    cdry[1, 0, 0] = np.nan
    cwet[-1, -1, -1] = np.inf
    g.upload_state(c, cdry, cwet, st["erumass"], st["outmass"], st["cd"])
    assert g.count_nonfinite() == (3, 2)
    # the count reads the state as it is now, it does not accumulate
    g.upload_state(f["c"], f["cdry"], f["cwet"], st["erumass"], st["outmass"], st["cd"])
    assert g.count_nonfinite() == (0, 0)
    g.close()
