"""The advection sweeps' slope limiter on special values, through the
fine-grained entry points, against the oracle bit for bit.

The binary64 sweeps evaluate the limiter of advctx.f90:34-40 (and advcty,
advctzc) on the bit patterns (sign and minimum as integer operations, one
division by dx instead of two); these fields put every case of that logic
in the differences the limiter sees: signed zeros, equal magnitudes of
either sign, subnormals, values whose differences overflow, infinities and
NaNs, and a non-positive dx (the reference's two divisions)."""
import numpy as np
import pytest

import fall3d_gb300 as F
import oracle_lib as O
from helpers import assert_same_bits

pytestmark = pytest.mark.gpu

NX, NY, NZ = 9, 8, 7
SPECIAL = np.array([0.0, -0.0, 1.0, -1.0, 2.0, 3.0, 1.5, 0.5, 1e-310, -1e-310, 5e-324, 1e308, -1e308,
                    1.7e308, np.inf, -np.inf, np.nan])


def _fields(seed, with_nonfinite):
    rng = np.random.default_rng(seed)
    shape = (NZ + 2, NY + 2, NX + 2)
    pool = SPECIAL if with_nonfinite else SPECIAL[np.isfinite(SPECIAL)]
    c = rng.choice(pool, size=shape)
    # arithmetic runs (|dr| == |dl|, same sign) and mirrored triples
    # (|dr| == |dl|, opposite signs) along every axis
    c[:, :, 1:4] = np.array([1.0, 2.0, 3.0])
    c[:, 2:5, :] = np.array([4.0, 1.0, 4.0])[None, :, None]
    c[2:5] = np.array([-1.0, -2.0, -3.0])[:, None, None]
    c[:, 6, 6] = -0.0
    vel = rng.choice([-2.0, -0.5, 0.0, -0.0, 0.5, 2.0], size=(NZ, NY, NX))
    vset = -np.abs(rng.uniform(0.0, 1.0, size=(NZ, NY, NX)))
    dz = rng.uniform(200.0, 800.0, size=NZ + 1)
    return np.ascontiguousarray(c), np.ascontiguousarray(vel), np.ascontiguousarray(vset), dz


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("nonfinite", [False, True])
@pytest.mark.parametrize("dx", [0.37, 1e-300, -0.25, 0.0])
@pytest.mark.parametrize("axis", ["x", "y"])
def test_horizontal_limiter(seed, nonfinite, dx, axis):
    c, vel, _, _ = _fields(seed, nonfinite)
    a, b = c.copy(), c.copy()
    args = (NX, NY, NZ, NZ, 1)
    dt = 7.5
    with np.errstate(all="ignore"):
        if axis == "x":
            O.load().orc_advctx(O.p(a), *args, O.p(vel), dx, dt)
            F.advctx(b, *args, vel, dx, dt)
        else:
            O.load().orc_advcty(O.p(a), *args, O.p(vel), dx, dt)
            F.advcty(b, *args, vel, dx, dt)
    assert_same_bits(b, a, f"advct{axis} dx={dx}")


@pytest.mark.parametrize("seed", [4, 5, 6])
@pytest.mark.parametrize("nonfinite", [False, True])
def test_vertical_limiter(seed, nonfinite):
    c, vel, vset, dz = _fields(seed, nonfinite)
    a, b = c.copy(), c.copy()
    args = (NX, NY, NZ, NZ, 1)
    dt = 3.25
    with np.errstate(all="ignore"):
        O.load().orc_advctzc(O.p(a), *args, O.p(vel), O.p(vset), O.p(dz), dt)
        F.advctzc(b, *args, vel, vset, dz, dt)
    assert_same_bits(b, a, "advctzc")
