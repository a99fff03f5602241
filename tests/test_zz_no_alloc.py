"""f3d_cmass2d_noalloc: the allocation-free variant of f3d_cmass2d (its
reduction scratch is a fixed device array compiled into the library) gives
the same outflow as f3d_cmass2d, called twice in a row through the C ABI,
over full and partial class and level ranges.

This file is collected last so that it also runs after every other test in
the same process (the fixed array is then reused, not fresh)."""
import ctypes as C

import numpy as np
import pytest

import fall3d_gb300 as F
import oracle_lib as O
from helpers import oracle_state

pytestmark = pytest.mark.gpu

# the same kernels and the same block count as f3d_cmass2d: only the
# summation order of the double-double partials could differ
RTOL = 1e-14
# against the oracle's sequential sum: (number of terms) * u relative to the
# sum of the absolute terms, with a wide margin
RTOL_ORACLE = 1e-13

VP, IP, DP = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)


def _lib():
    lib = F.load()
    fn = lib.f3d_cmass2d_noalloc
    fn.argtypes = [VP, VP, VP, VP, VP, IP, IP, IP, IP, IP, IP, IP, IP, DP, DP, VP, DP, DP]
    fn.restype = C.c_int
    return lib


def _fields(s, o, seed):
    f, co, g = o.fields(), o.coeffs(), s.grid
    # a positive field everywhere (ghosts included) so every face carries flux
    c = np.random.default_rng(seed).random(f["c"].shape)
    return dict(c=np.ascontiguousarray(c), vx=co["vx"], vy=co["vy"], vz=co["vz"],
                vset=np.ascontiguousarray(f["vset"]), dz=np.ascontiguousarray(g["dz"]),
                nx=g["nx"], ny=g["ny"], nz=g["nz"], nc=g["nc"], dX1=g["dX1"], dX2=g["dX2"],
                dt=o.state()["dt"])


@pytest.fixture(scope="module")
def case():
    s, o = oracle_state("small", seed=5, steps=1)
    return _fields(s, o, 11)


@pytest.fixture(scope="module")
def wide():
    """96 x 80 x 20: 14720 face cells, so the reduction takes 58 blocks."""
    s, o = oracle_state("small", seed=6, steps=0, nx=96, ny=80, nz=20, nc=3)
    return _fields(s, o, 12)


def _device(k):
    torch = pytest.importorskip("torch")
    t = {n: torch.from_numpy(np.ascontiguousarray(k[n])).cuda() for n in ("c", "vx", "vy", "vz", "vset", "dz")}
    torch.cuda.synchronize()
    return t, {n: C.c_void_p(v.data_ptr()) for n, v in t.items()}


def _noalloc(lib, dev, k, outmass, rng=None):
    ic, ncl, iz, nzl = rng if rng is not None else (1, k["nc"], 1, k["nz"])
    i = lambda v: C.byref(C.c_int(int(v)))
    d = lambda v: C.byref(C.c_double(float(v)))
    om = C.c_double(outmass)
    rc = lib.f3d_cmass2d_noalloc(dev["c"], dev["vx"], dev["vy"], dev["vz"], dev["vset"], i(k["nx"]),
                                 i(k["ny"]), i(k["nz"]), i(k["nc"]), i(ic), i(ncl), i(iz), i(nzl),
                                 d(k["dX1"]), d(k["dX2"]), dev["dz"], d(k["dt"]), C.byref(om))
    return rc, om.value


def _args(k, rng):
    ic, ncl, iz, nzl = rng
    return (k["vx"], k["vy"], k["vz"], k["vset"], k["nx"], k["ny"], k["nz"], k["nc"], ic, ncl, iz, nzl,
            k["dX1"], k["dX2"], k["dz"], k["dt"])


def _oracle(k, rng, outmass, vabs=False):
    """The oracle's outflow; with vabs every velocity is |v| and c >= 0, so
    every term is non-negative and the result is the sum of |terms|."""
    v = {n: np.abs(k[n]) if vabs else k[n] for n in ("vx", "vy", "vz", "vset")}
    om = np.array([outmass])
    ic, ncl, iz, nzl = rng
    O.load().orc_cmass2d(O.p(k["c"]), O.p(v["vx"]), O.p(v["vy"]), O.p(v["vz"]), O.p(v["vset"]), k["nx"],
                         k["ny"], k["nz"], k["nc"], ic, ncl, iz, nzl, k["dX1"], k["dX2"], O.p(k["dz"]),
                         k["dt"], O.p(om))
    return om[0]


def _ranges(k):
    nc, nz = k["nc"], k["nz"]
    return [(1, nc, 1, nz),            # everything
            (2, nc - 1, 1, nz),        # a class offset
            (1, nc, 1, nz - 3),        # the top face absent
            (2, 2, 4, nz - 3),         # a z slab that owns the top face
            (1, 0, 1, nz)]             # no classes: outmass unchanged


def test_noalloc_matches_cmass2d_twice(case):
    lib = _lib()
    k = case
    _t, dev = _device(k)
    for rng in _ranges(k):
        # the existing entry point, twice in a row (outmass accumulates)
        ref1 = F.cmass2d(k["c"], *_args(k, rng), 7.0)
        ref2 = F.cmass2d(k["c"], *_args(k, rng), ref1)
        rc1, got1 = _noalloc(lib, dev, k, 7.0, rng)
        assert rc1 == 0, F.last_error()
        rc2, got2 = _noalloc(lib, dev, k, got1, rng)
        assert rc2 == 0, F.last_error()
        assert abs(got1 - ref1) <= RTOL * abs(ref1), (rng, got1, ref1)
        assert abs(got2 - ref2) <= RTOL * abs(ref2), (rng, got2, ref2)
        # and both against the oracle's sequential sum
        orc = _oracle(k, rng, 7.0)
        scale = _oracle(k, rng, 0.0, vabs=True) + 7.0
        assert abs(got1 - orc) <= RTOL_ORACLE * scale, (rng, got1, orc)
        if rng[1] == 0:
            assert got1 == 7.0 and got2 == 7.0 and ref1 == 7.0
        else:
            assert abs(ref1 - 7.0) > 1.0  # a non-trivial net flux through the faces


def test_noalloc_no_classes_on_a_wide_grid(wide):
    """nc_loc = 0 with more face cells than one block's share: the block
    partials must not reach the outmass accumulator."""
    lib = _lib()
    k = wide
    _t, dev = _device(k)
    for outmass in (3.25, -1.5e6):
        rc, got = _noalloc(lib, dev, k, outmass, (1, 0, 1, k["nz"]))
        assert rc == 0, F.last_error()
        assert got == outmass
        assert F.cmass2d(k["c"], *_args(k, (1, 0, 1, k["nz"])), outmass) == outmass
    full = (1, k["nc"], 1, k["nz"])
    rc, got = _noalloc(lib, dev, k, 0.5, full)
    assert rc == 0, F.last_error()
    ref = F.cmass2d(k["c"], *_args(k, full), 0.5)
    assert abs(got - ref) <= RTOL * abs(ref)


def test_noalloc_rejects_host_arrays(case):
    lib = _lib()
    k = case
    host = {n: C.c_void_p(k[n].ctypes.data) for n in ("c", "vx", "vy", "vz", "vset", "dz")}
    rc, _ = _noalloc(lib, host, k, 0.0)
    assert rc == 1  # F3D_ERR_ARG
    assert "device" in F.last_error()
