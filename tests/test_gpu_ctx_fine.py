"""One plain-form context step against the same step assembled from the
fine-grained entry points, class by class, on the context's own
coefficients: bit for bit.

The context's sweeps take each line through all classes, read 1/rho, rkh*rho
and the diffz face coefficients formed once per meteo update, and form
diffz's c/rho from 1/rho (Markstein's correction); the fine-grained routines
run one class in the reference's operation order with the IEEE division and
are bit for bit equal to the oracle (tests/test_gpu_fine.py).  So this pins the context's transport to
the oracle's on the same coefficients (Sources/sizloop.f90:31-83)."""
import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import synth
from helpers import assert_same_bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,steps,wet", [(5, 8, False), (6, 9, False), (7, 8, True)])  # both x/y orders
def test_context_step_equals_fine_grained_sequence(seed, steps, wet):
    s = synth.make_scenario("small", seed=seed, wetdep=wet)
    gr = s.grid
    nx, ny, nz, nc = gr["nx"], gr["ny"], gr["nz"], gr["nc"]
    # a plume to transport
    g0 = F.Context(s, F.PREC_FP64)
    g0.run(max_steps=steps)
    f0 = g0.fields()
    g0.close()
    assert np.max(f0["c"]) > 0.0

    g = F.Context(s, F.PREC_FP64)
    g.meteo(0)  # no source interval is loaded: setsrc adds nothing
    g.upload_state(c=f0["c"], cdry=f0["cdry"], cwet=f0["cwet"])
    g.set_time(g.state()["time"], steps)  # the iiter parity of the compared step
    st = g.state()
    co, fl = g.coeffs(), g.fields()
    g.step()
    g.sync()
    want = g.fields()
    g.close()

    dt, it = st["dt"], st["iiter"] + 1
    dz = np.ascontiguousarray(gr["dz"], dtype=np.float64)
    c = fl["c"].copy()
    cdry = fl["cdry"].copy()
    cwet = fl["cwet"].copy()
    # the context's wet inputs: PBLH as read, PRATE in mm/h (reamet.f90:146)
    zi = np.ascontiguousarray(s.met["pblh"][0], dtype=np.float64)
    prate = np.ascontiguousarray(s.met["prate"][0], dtype=np.float64) * 3600.0
    zlayer = np.ascontiguousarray(gr["zlayer"], dtype=np.float64)
    diam = np.ascontiguousarray(gr["diam"], dtype=np.float64)
    args = (nx, ny, nz, nz, 1)
    for ic in range(nc):
        cc = np.ascontiguousarray(c[ic])
        vs, vd = np.ascontiguousarray(fl["vset"][ic]), np.ascontiguousarray(fl["vdep"][ic])
        F.setbcc(cc, *args, co["vx"], co["vy"], co["vz"], vs, vd, co["rkver"], dz)
        F.advctzc(cc, *args, co["vz"], vs, dz, dt)
        advx = lambda: F.advctx(cc, *args, co["vx"], gr["dX1"], dt)
        advy = lambda: F.advcty(cc, *args, co["vy"], gr["dX2"], dt)
        (advx(), advy()) if it % 2 == 0 else (advy(), advx())
        F.diffz(cc, *args, dz, dt, co["rkver"], co["rho"])
        difx = lambda: F.diffx(cc, *args, gr["dX1"], dt, co["rkh1"], co["rho"])
        dify = lambda: F.diffy(cc, *args, gr["dX2"], dt, co["rkhor"], co["rho"])
        (difx(), dify()) if it % 2 == 0 else (dify(), difx())
        if wet and ic < gr["np"]:
            F.wetdep(cc, cwet, ic + 1, *args, dt, diam, zlayer, dz, zi, prate)
        F.accum(cc, cdry, ic + 1, *args, co["vz"], dt, vs, vd)
        c[ic] = cc
    F.clip(c, nx, ny, nz, nc)
    assert_same_bits(want["c"], c, "c")
    assert_same_bits(want["cdry"], cdry, "cdry")
    assert_same_bits(want["cwet"], cwet, "cwet")
    if wet:
        assert np.max(want["cwet"]) > np.max(fl["cwet"])  # the step deposited
