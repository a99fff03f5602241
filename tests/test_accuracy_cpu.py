"""The storage-rounding bound of fall3d_gb300/accuracy.py: the relative
standard deviation of rounding binary64 values to binary32 (SIGMA_U) and
the effective number of mass-carrying cells N_eff; the error that rounding
adds to a total of N_eff equal masses is SIGMA_U / sqrt(N_eff)."""
import numpy as np

from fall3d_gb300 import accuracy


def test_sigma_u_is_the_rounding_spread():
    rng = np.random.default_rng(5)
    x = np.exp(rng.uniform(np.log(1e-12), np.log(1e3), 2_000_000))
    rel = (x.astype(np.float32).astype(np.float64) - x) / x
    assert abs(rel.mean()) < 0.01 * accuracy.SIGMA_U
    assert abs(rel.std() / accuracy.SIGMA_U - 1.0) < 0.02
    assert np.max(np.abs(rel)) <= accuracy.U32


def test_n_eff_and_the_total_of_rounded_masses():
    nc, nz, ny, nx = 2, 4, 30, 40
    dz = np.ones(nz + 1)
    c = np.zeros((nc, nz + 2, ny + 2, nx + 2))
    c[:, 1:-1, 1:-1, 1:-1] = 1.0
    assert abs(accuracy._n_eff(c, dz) - nc * nz * ny * nx) < 1e-6
    one = np.zeros_like(c)
    one[1, 2, 3, 4] = 7.0
    assert abs(accuracy._n_eff(one, dz) - 1.0) < 1e-12
    # the spread of the total after rounding every cell once
    rng = np.random.default_rng(9)
    m = np.exp(rng.normal(0.0, 2.0, (400, 5000)))
    tot = m.sum(axis=1)
    err = (m.astype(np.float32).astype(np.float64).sum(axis=1) - tot) / tot
    n_eff = tot ** 2 / np.square(m).sum(axis=1)
    pred = accuracy.SIGMA_U / np.sqrt(n_eff)
    assert 0.7 < np.sqrt(np.mean((err / pred) ** 2)) < 1.3
