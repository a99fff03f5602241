import numpy as np
import pytest

from fall3d_gb300 import synth


def test_generator_is_seeded():
    a = synth.make_scenario("tiny", seed=5)
    b = synth.make_scenario("tiny", seed=5)
    c = synth.make_scenario("tiny", seed=6)
    assert np.array_equal(a.met["u"], b.met["u"])
    assert not np.array_equal(a.met["u"], c.met["u"])


def test_met_fields_are_float32_values():
    s = synth.make_scenario("small", seed=1)
    for k in ("u", "v", "t", "tp", "rho", "ust", "pblh", "rmol", "znt", "prate"):
        a = s.met[k]
        assert np.array_equal(a, a.astype(np.float32).astype(np.float64)), k


def test_grid_follows_reagrd():
    s = synth.make_scenario("cfg0", seed=0)
    g = s.grid
    assert (g["nx"], g["ny"], g["nz"], g["nc"]) == (80, 80, 25, 6)
    assert g["dz"][0] == g["dz"][1] and g["dz"][-1] == g["dz"][-2]
    assert np.allclose(g["dX1"], synth.REARTH * 0.05 * synth.PI / 180.0)
    assert np.all((g["Hm1"] > 0) & (g["Hm1"] <= 1))


def test_source_mass_matches_mer():
    s = synth.make_scenario("cfg0", seed=0)
    n = s.src["nsou"][0]
    tot = s.src["tmrat"][: n * s.grid["nc"]].sum()
    assert abs(tot - 1e6) / 1e6 < 1e-6
    assert s.src["nsou"][1] == 0


def test_classes_and_fractions():
    cls = synth.make_classes(6, -1.0, 4.0)
    assert abs(cls["fc"].sum() - 1.0) < 1e-12
    assert np.allclose(cls["diam"] * 1e3, 2.0 ** -np.linspace(-1, 4, 6), rtol=1e-6)
    agg = synth.make_classes(5, 0.0, 4.0, aggregate=(0.2, 1000.0, 0.2))
    assert agg["names"][-1] == "aggregate" and abs(agg["fc"].sum() - 1.0) < 1e-12


@pytest.mark.parametrize("seed", [0, 3])
def test_ensemble_member_bounds(seed):
    s = synth.ensemble_member(seed, run_h=1.0, max_snapshots=2)
    g = s.grid
    assert 64 <= g["nx"] <= 320 and 64 <= g["ny"] <= 320 and 20 <= g["nz"] <= 60
    assert 4 <= g["nc"] <= 20
