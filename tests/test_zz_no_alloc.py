"""f3d_cmass2d_noalloc: the allocation-free variant of f3d_cmass2d (its
reduction scratch is a fixed device array compiled into the library) gives
the same outflow as f3d_cmass2d, called twice in a row through the C ABI.

This file is collected last so that it also runs after every other test in
the same process (the fixed array is then reused, not fresh)."""
import ctypes as C

import numpy as np
import pytest

import fall3d_gb300 as F
from helpers import oracle_state

pytestmark = pytest.mark.gpu

# the same reduction over the same terms: only the summation order of the
# double-double partials could differ, so the two results agree to a few ulp
RTOL = 1e-14

VP, IP, DP = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)


def _lib():
    lib = F.load()
    fn = lib.f3d_cmass2d_noalloc
    fn.argtypes = [VP, VP, VP, VP, VP, IP, IP, IP, IP, IP, IP, IP, IP, DP, DP, VP, DP, DP]
    fn.restype = C.c_int
    return lib


@pytest.fixture(scope="module")
def case():
    s, o = oracle_state("small", seed=5, steps=1)
    f, co, g = o.fields(), o.coeffs(), s.grid
    # a positive field everywhere (ghosts included) so every face carries flux
    c = np.random.default_rng(11).random(f["c"].shape)
    return dict(c=np.ascontiguousarray(c), vx=co["vx"], vy=co["vy"], vz=co["vz"],
                vset=np.ascontiguousarray(f["vset"]), dz=np.ascontiguousarray(g["dz"]),
                nx=g["nx"], ny=g["ny"], nz=g["nz"], nc=g["nc"], dX1=g["dX1"], dX2=g["dX2"],
                dt=o.state()["dt"])


def _noalloc(lib, dev, k, outmass):
    i = lambda v: C.byref(C.c_int(int(v)))
    d = lambda v: C.byref(C.c_double(float(v)))
    om = C.c_double(outmass)
    rc = lib.f3d_cmass2d_noalloc(dev["c"], dev["vx"], dev["vy"], dev["vz"], dev["vset"], i(k["nx"]),
                                 i(k["ny"]), i(k["nz"]), i(k["nc"]), i(1), i(k["nc"]), i(1), i(k["nz"]),
                                 d(k["dX1"]), d(k["dX2"]), dev["dz"], d(k["dt"]), C.byref(om))
    return rc, om.value


def test_noalloc_matches_cmass2d_twice(case):
    torch = pytest.importorskip("torch")
    lib = _lib()
    k = case
    t = {n: torch.from_numpy(np.ascontiguousarray(k[n])).cuda() for n in ("c", "vx", "vy", "vz", "vset", "dz")}
    torch.cuda.synchronize()
    dev = {n: C.c_void_p(v.data_ptr()) for n, v in t.items()}
    args = (k["vx"], k["vy"], k["vz"], k["vset"], k["nx"], k["ny"], k["nz"], k["nc"], 1, k["nc"], 1, k["nz"],
            k["dX1"], k["dX2"], k["dz"], k["dt"])
    # the existing entry point, twice in a row (outmass accumulates)
    ref1 = F.cmass2d(k["c"], *args, 7.0)
    ref2 = F.cmass2d(k["c"], *args, ref1)
    assert abs(ref1 - 7.0) > 1.0  # a non-trivial net flux through the boundary faces
    rc1, got1 = _noalloc(lib, dev, k, 7.0)
    assert rc1 == 0, F.last_error()
    rc2, got2 = _noalloc(lib, dev, k, got1)
    assert rc2 == 0, F.last_error()
    assert abs(got1 - ref1) <= RTOL * abs(ref1), (got1, ref1)
    assert abs(got2 - ref2) <= RTOL * abs(ref2), (got2, ref2)


def test_noalloc_rejects_host_arrays(case):
    lib = _lib()
    k = case
    host = {n: C.c_void_p(k[n].ctypes.data) for n in ("c", "vx", "vy", "vz", "vset", "dz")}
    rc, _ = _noalloc(lib, host, k, 0.0)
    assert rc == 1  # F3D_ERR_ARG
    assert "device" in F.last_error()
