"""Per-routine parity of the CUDA fine-grained entry points against the CPU
oracle on the same plume-bearing state.

Routines built only from +,-,*,/,sqrt, comparisons and the fixed MAX/MIN/
SIGN semantics must agree bit for bit (NaN payloads aside).  Routines that
call pow/log/exp/atan/acos/tan (wetdep, kappa3 RAMS, setvset, setvdrydep)
agree to a few ulp; the budget sums (cmass2d, cmass3d) differ by the order
of summation only.  Tolerances are written in each test.
"""
import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import synth
import oracle_lib as O
from helpers import oracle_state, assert_same_bits, assert_close

pytestmark = pytest.mark.gpu

RTOL_LIBM = 1e-13  # CUDA vs host libm, propagated through a few operations


@pytest.fixture(scope="module")
def st():
    s, o = oracle_state("small", seed=3, steps=6)
    f = o.fields()
    co = o.coeffs()
    g = s.grid
    return dict(s=s, o=o, f=f, co=co, g=g, nx=g["nx"], ny=g["ny"], nz=g["nz"], nc=g["nc"])


def _cls(st, ic):
    f, co, g = st["f"], st["co"], st["g"]
    return dict(c=np.ascontiguousarray(f["c"][ic]), vset=np.ascontiguousarray(f["vset"][ic]),
                vdep=np.ascontiguousarray(f["vdep"][ic]))


def _with_bcc(st, ic, nz_loc=None, iz_loc=1):
    """Class ic's field after the oracle's setbcc (realistic ghosts, incl.
    the non-finite SIMILARITY bottom ghosts)."""
    lib = O.load()
    k = _cls(st, ic)
    co, g = st["co"], st["g"]
    nz_loc = st["nz"] if nz_loc is None else nz_loc
    lib.orc_setbcc(O.p(k["c"]), st["nx"], st["ny"], st["nz"], nz_loc, iz_loc, O.p(co["vx"]),
                   O.p(co["vy"]), O.p(co["vz"]), O.p(k["vset"]), O.p(k["vdep"]), O.p(co["rkver"]),
                   O.p(g["dz"]))
    return k


@pytest.mark.parametrize("zr", [None, (5, 4), (3, 1)])
def test_setbcc(st, zr):
    nz_loc, iz_loc = (st["nz"], 1) if zr is None else zr
    k = _cls(st, 1)
    co, g = st["co"], st["g"]
    a = k["c"].copy()
    b = k["c"].copy()
    args = (st["nx"], st["ny"], st["nz"], nz_loc, iz_loc)
    O.load().orc_setbcc(O.p(a), *args, O.p(co["vx"]), O.p(co["vy"]), O.p(co["vz"]), O.p(k["vset"]),
                        O.p(k["vdep"]), O.p(co["rkver"]), O.p(g["dz"]))
    F.setbcc(b, *args, co["vx"], co["vy"], co["vz"], k["vset"], k["vdep"], co["rkver"], g["dz"])
    assert_same_bits(b, a, "setbcc")
    if zr is None:
        assert np.isnan(a).any() or np.isinf(a).any()  # the SIMILARITY ghosts are exercised


@pytest.mark.parametrize("ic", [0, 3])
@pytest.mark.parametrize("zr", [None, (6, 4)])
def test_advctzc(st, ic, zr):
    nz_loc, iz_loc = (st["nz"], 1) if zr is None else zr
    k = _with_bcc(st, ic)
    co, g = st["co"], st["g"]
    a, b = k["c"].copy(), k["c"].copy()
    dt = st["o"].state()["dt"]
    args = (st["nx"], st["ny"], st["nz"], nz_loc, iz_loc)
    O.load().orc_advctzc(O.p(a), *args, O.p(co["vz"]), O.p(k["vset"]), O.p(g["dz"]), dt)
    F.advctzc(b, *args, co["vz"], k["vset"], g["dz"], dt)
    assert_same_bits(b, a, "advctzc")


@pytest.mark.parametrize("axis", ["x", "y"])
@pytest.mark.parametrize("zr", [None, (4, 3)])
def test_advection_xy(st, axis, zr):
    nz_loc, iz_loc = (st["nz"], 1) if zr is None else zr
    k = _with_bcc(st, 2)
    co, g = st["co"], st["g"]
    a, b = k["c"].copy(), k["c"].copy()
    dt = st["o"].state()["dt"]
    args = (st["nx"], st["ny"], st["nz"], nz_loc, iz_loc)
    if axis == "x":
        O.load().orc_advctx(O.p(a), *args, O.p(co["vx"]), g["dX1"], dt)
        F.advctx(b, *args, co["vx"], g["dX1"], dt)
    else:
        O.load().orc_advcty(O.p(a), *args, O.p(co["vy"]), g["dX2"], dt)
        F.advcty(b, *args, co["vy"], g["dX2"], dt)
    assert_same_bits(b, a, f"advct{axis}")


@pytest.mark.parametrize("zr", [None, (5, 5), (2, 3)])
def test_diffz(st, zr):
    nz_loc, iz_loc = (st["nz"], 1) if zr is None else zr
    k = _with_bcc(st, 1)
    co, g = st["co"], st["g"]
    a, b = k["c"].copy(), k["c"].copy()
    dt = st["o"].state()["dt"]
    args = (st["nx"], st["ny"], st["nz"], nz_loc, iz_loc)
    O.load().orc_diffz(O.p(a), *args, O.p(g["dz"]), dt, O.p(co["rkver"]), O.p(co["rho"]))
    F.diffz(b, *args, g["dz"], dt, co["rkver"], co["rho"])
    assert_same_bits(b, a, "diffz")


@pytest.mark.parametrize("axis", ["x", "y"])
def test_diffusion_xy(st, axis):
    k = _with_bcc(st, 0)
    co, g = st["co"], st["g"]
    a, b = k["c"].copy(), k["c"].copy()
    dt = st["o"].state()["dt"]
    args = (st["nx"], st["ny"], st["nz"], st["nz"], 1)
    if axis == "x":
        O.load().orc_diffx(O.p(a), *args, g["dX1"], dt, O.p(co["rkh1"]), O.p(co["rho"]))
        F.diffx(b, *args, g["dX1"], dt, co["rkh1"], co["rho"])
    else:
        O.load().orc_diffy(O.p(a), *args, g["dX2"], dt, O.p(co["rkhor"]), O.p(co["rho"]))
        F.diffy(b, *args, g["dX2"], dt, co["rkhor"], co["rho"])
    assert_same_bits(b, a, f"diff{axis}")


def test_device_pointer_path_matches_host_path(st):
    torch = pytest.importorskip("torch")
    k = _with_bcc(st, 3)
    co, g = st["co"], st["g"]
    dt = st["o"].state()["dt"]
    args = (st["nx"], st["ny"], st["nz"], st["nz"], 1)
    a = k["c"].copy()
    F.advctx(a, *args, co["vx"], g["dX1"], dt)
    F.diffz(a, *args, g["dz"], dt, co["rkver"], co["rho"])
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    b = dev(k["c"])
    F.advctx(b, *args, dev(co["vx"]), g["dX1"], dt)
    F.diffz(b, *args, dev(g["dz"]), dt, dev(co["rkver"]), dev(co["rho"]))
    assert_same_bits(b.cpu().numpy(), a, "device path")
    with pytest.raises(F.F3DError):  # mixing host and device arrays is rejected
        F.advctx(b, *args, co["vx"], g["dX1"], dt)


def test_wetdep_and_accum(st):
    lib = O.load()
    co, g = st["co"], st["g"]
    nx, ny, nz, nc = st["nx"], st["ny"], st["nz"], st["nc"]
    rng = np.random.default_rng(7)
    prate = np.ascontiguousarray(rng.uniform(0.0, 5.0, (ny, nx)))  # mm/h
    zi = np.ascontiguousarray(rng.uniform(500.0, 3000.0, (ny, nx)))
    dt = st["o"].state()["dt"]
    for ic in range(1, nc + 1):
        k = _with_bcc(st, ic - 1)
        a, b = k["c"].copy(), k["c"].copy()
        wa = np.ascontiguousarray(rng.random((nc + 1, ny, nx)))
        wb = wa.copy()
        lib.orc_wetdep(O.p(a), O.p(wa), ic, nx, ny, nz, nz, 1, dt, O.p(g["diam"]), O.p(g["zlayer"]),
                       O.p(g["dz"]), O.p(zi), O.p(prate))
        F.wetdep(b, wb, ic, nx, ny, nz, nz, 1, dt, g["diam"], g["zlayer"], g["dz"], zi, prate)
        assert_close(b, a, RTOL_LIBM, 0.0, f"wetdep c class {ic}")
        assert_close(wb, wa, RTOL_LIBM, 0.0, f"wetdep cwet class {ic}")
        da = np.ascontiguousarray(rng.random((nc + 1, ny, nx)))
        db = da.copy()
        lib.orc_accum(O.p(a), O.p(da), ic, nx, ny, nz, nz, 1, dt, O.p(k["vset"]),
                      O.p(np.ascontiguousarray(k["vdep"] - 0.01)))
        F.accum(a, db, ic, nx, ny, nz, nz, 1, co["vz"], dt, k["vset"],
                np.ascontiguousarray(k["vdep"] - 0.01))
        assert_same_bits(db, da, f"accum class {ic}")


def test_clip_and_cmass(st):
    lib = O.load()
    co, g, f = st["co"], st["g"], st["f"]
    nx, ny, nz, nc = st["nx"], st["ny"], st["nz"], st["nc"]
    c = np.ascontiguousarray(f["c"]).copy()
    for ic in range(nc):  # fresh ghosts for every class, then perturb below zero
        k = _with_bcc(st, ic)
        c[ic] = k["c"]
    c[:, 2:5, 3:6, 4:9] -= 1e-3
    a, b = c.copy(), c.copy()
    lib.orc_clip(O.p(a), nx, ny, nz, 1, nc)
    F.clip(b, nx, ny, nz, nc)
    assert_same_bits(b, a, "clip")
    vset = np.ascontiguousarray(f["vset"])
    dt = st["o"].state()["dt"]
    om = np.array([123.0])
    lib.orc_cmass2d(O.p(a), O.p(co["vx"]), O.p(co["vy"]), O.p(co["vz"]), O.p(vset), nx, ny, nz, nc, 1,
                    nc, 1, nz, g["dX1"], g["dX2"], O.p(g["dz"]), dt, O.p(om))
    omg = F.cmass2d(b, co["vx"], co["vy"], co["vz"], vset, nx, ny, nz, nc, 1, nc, 1, nz, g["dX1"],
                    g["dX2"], g["dz"], dt, 123.0)
    # summation order only: all terms >= 0, so the bound (N-1)u is relative
    assert abs(omg - om[0]) <= 1e-13 * abs(om[0])
    cl = np.ascontiguousarray(np.abs(np.random.default_rng(1).random((nc + 1, ny, nx))))
    out = np.zeros(4)
    lib.orc_cmass3d(O.p(a), O.p(cl), O.p(cl), O.p(cl), nx, ny, nz, nc, g["dX1"], g["dX2"], O.p(g["dz"]),
                    O.p(out))
    got = F.cmass3d(b, cl, cl, cl, nx, ny, nz, nc, g["dX1"], g["dX2"], g["dz"])
    for x, y, nm in zip(got, out, ("massvol", "massdep", "massdry", "masswet")):
        assert abs(x - y) <= 1e-13 * abs(y), nm


def test_getc0(st):
    nx, ny, nc = st["nx"], st["ny"], st["nc"]
    rng = np.random.default_rng(2)
    d0 = np.ascontiguousarray(rng.random((nc + 1, ny, nx)))
    w0 = np.ascontiguousarray(rng.random((nc + 1, ny, nx)))
    da, wa, la = d0.copy(), w0.copy(), np.zeros_like(d0)
    db, wb, lb = d0.copy(), w0.copy(), np.zeros_like(d0)
    O.load().orc_getc0(O.p(da), O.p(wa), O.p(la), nx, ny, nc, nc - 1)
    F.getc0(db, wb, lb, nx, ny, nc, nc - 1)
    for x, y, nm in ((db, da, "cdry"), (wb, wa, "cwet"), (lb, la, "cload")):
        assert_same_bits(x, y, nm)


def test_setsrc(st):
    g = st["g"]
    nx, ny, nz, nc = st["nx"], st["ny"], st["nz"], st["nc"]
    rng = np.random.default_rng(4)
    n = 40
    isrc = rng.integers(1, nx + 1, n).astype(np.int32)
    jsrc = rng.integers(1, ny + 1, n).astype(np.int32)
    ksrc = rng.integers(0, nz + 1, n).astype(np.int32)  # k = 0 is skipped, as in the reference
    isrc[5:9] = isrc[4]
    jsrc[5:9] = jsrc[4]
    ksrc[5:9] = ksrc[4]  # several sources in one cell add in order
    tm = np.ascontiguousarray(rng.random(n * nc) * 1e5)
    c = np.ascontiguousarray(st["f"]["c"]).copy()
    a, b = c.copy(), c.copy()
    dt = 13.7
    rc = O.load().orc_setsrc(O.p(a), nx, ny, nz, nc, n, O.ip(isrc), O.ip(jsrc), O.ip(ksrc), O.p(tm),
                             O.p(g["dz"]), O.p(g["zlayer"]), O.p(g["Hm1"]), g["dX1"], g["dX2"], dt)
    assert rc == 0
    F.setsrc(b, nx, ny, nz, nc, n, isrc, jsrc, ksrc, tm, g["dz"], g["zlayer"], g["Hm1"], g["dX1"],
             g["dX2"], dt)
    assert_same_bits(b, a, "setsrc")
    bad = isrc.copy()
    bad[3] = nx + 1
    with pytest.raises(F.F3DError):
        F.setsrc(b, nx, ny, nz, nc, n, bad, jsrc, ksrc, tm, g["dz"], g["zlayer"], g["Hm1"], g["dX1"],
                 g["dX2"], dt)


def test_finddt(st):
    co, g, f = st["co"], st["g"], st["f"]
    nx, ny, nz, nc = st["nx"], st["ny"], st["nz"], st["nc"]
    vset = np.ascontiguousarray(f["vset"])
    out = np.zeros(2)
    O.load().orc_finddt(nx, ny, nz, nc, g["dX1"], g["dX2"], O.p(g["dz"]), O.p(co["vx"]), O.p(co["vy"]),
                        O.p(co["vz"]), O.p(vset), O.p(co["rkh1"]), O.p(co["rkhor"]), O.p(co["rkver"]),
                        0.9, O.p(out[:1]), O.p(out[1:]))
    dt, dtc = F.finddt(nx, ny, nz, nc, g["dX1"], g["dX2"], g["dz"], co["vx"], co["vy"], co["vz"], vset,
                       co["rkh1"], co["rkhor"], co["rkver"], 0.9)
    assert_same_bits(np.array([dt, dtc]), out, "finddt")


@pytest.mark.parametrize("modkv,modkh,coord", [(1, 1, 0), (0, 0, 0), (2, 2, 0), (1, 2, 1), (2, 1, 1)])
def test_kappa3(modkv, modkh, coord):
    s = synth.make_scenario("small", seed=11, coord=coord, spacing=0.05 if coord == 0 else 4000.0,
                            rmol=-1.0 / 300.0 if modkv == 2 else 1.0 / 500.0, rkh0=321.0, rkv0=12.5)
    g, m = s.grid, s.met
    nx, ny, nz = g["nx"], g["ny"], g["nz"]
    f3 = {k: np.ascontiguousarray(m[k][0]) for k in ("u", "v", "tp")}
    f2 = {k: np.ascontiguousarray(m[k][0]) for k in ("ust", "pblh", "rmol")}
    f2["rmol"] = np.ascontiguousarray(f2["rmol"] * np.linspace(-1.0, 1.0, nx)[None, :])  # both stabilities
    outs = []
    for impl in ("oracle", "gpu"):
        kv = np.full((nz, ny, nx), 7.0)
        kh = np.full((nz, ny, nx), 7.0)
        if impl == "oracle":
            O.load().orc_kappa3(nx, ny, nz, modkv, modkh, coord, g["rkv0"], g["rkh0"], g["Csh"], g["dX1"],
                                g["dX2"], g["dx"], g["dy"], O.p(g["dz"]), O.p(g["zlayer"]), O.p(g["Hm1"]),
                                O.p(f3["u"]), O.p(f3["v"]), O.p(f3["tp"]), O.p(f2["ust"]), O.p(f2["pblh"]),
                                O.p(f2["rmol"]), O.p(kv), O.p(kh))
        else:
            F.kappa3(nx, ny, nz, modkv, modkh, coord, g["rkv0"], g["rkh0"], g["Csh"], g["dX1"], g["dX2"],
                     g["dx"], g["dy"], g["dz"], g["zlayer"], g["Hm1"], f3["u"], f3["v"], f3["tp"],
                     f2["ust"], f2["pblh"], f2["rmol"], kv, kh)
        outs.append((kv, kh))
    (kva, kha), (kvb, khb) = outs
    if modkv == 1:
        assert np.all(kva[0] == 7.0)  # k = 1 is not assigned under SIMILARITY
    # SIMILARITY/SURFACE use sqrt only: exact; RAMS's Kmh uses pow: a few ulp
    assert_same_bits(kvb, kva, "rkver")
    assert_close(khb, kha, RTOL_LIBM, 0.0, "rkhor")


@pytest.mark.parametrize("modv", [1, 2, 3, 4])
def test_setvset_chain(modv):
    s = synth.make_scenario("small", seed=5, nc=5)
    g, m = s.grid, s.met
    nx, ny, nz, nc = g["nx"], g["ny"], g["nz"], g["nc"]
    psi = g["psi"].copy()
    if modv == 3:
        psi = np.full(nc, 0.7)
    np_ = nc - 1  # last class is a gas: its vset keeps the alternating-sign zero
    T = np.ascontiguousarray(m["t"][0])
    R = np.ascontiguousarray(m["rho"][0])
    va = np.zeros((nc, nz, ny, nx))
    vb = np.zeros((nc, nz, ny, nx))
    cda = np.array([1.0])
    cdb = 1.0
    for upd in range(2):  # two meteo updates: the cd chain continues
        its = np.zeros((nc, nz, ny, nx), np.int32)
        rc = O.load().orc_setvset(nx, ny, nz, nc, np_, modv, O.p(g["diam"]), O.p(g["rhop"]), O.p(psi),
                                  O.p(g["sphe"]), O.p(T), O.p(R), 0, 1.0, O.p(va), O.p(cda), O.ip(its))
        assert rc == 0
        cdb = F.setvset(nx, ny, nz, nc, np_, modv, g["diam"], g["rhop"], psi, g["sphe"], T, R, 0, 1.0, vb,
                        cdb)
        assert_close(vb, va, RTOL_LIBM, 0.0, f"vset update {upd}")
        assert np.array_equal(np.signbit(vb[np_:]), np.signbit(va[np_:]))
        if modv != 4:
            assert abs(cdb - cda[0]) <= RTOL_LIBM * abs(cda[0])
        T = np.ascontiguousarray(T + 1.5)


def test_setvdrydep():
    s = synth.make_scenario("small", seed=8, nc=6, phimin=3.0, phimax=12.0)  # 125 um .. 0.24 um
    g, m = s.grid, s.met
    nx, ny, nc = g["nx"], g["ny"], g["nc"]
    rng = np.random.default_rng(9)
    zl = np.ascontiguousarray(g["zlayer"] + 10.0)  # first level above ground: finite ra
    ldu = np.ascontiguousarray(rng.integers(-2, 27, (ny, nx)).astype(np.float64))
    rl = np.ascontiguousarray(rng.uniform(-0.02, 0.02, (ny, nx)))
    znt = np.ascontiguousarray(rng.uniform(0.01, 1.0, (ny, nx)))
    ust = np.ascontiguousarray(rng.uniform(0.0, 0.6, (ny, nx)))
    ust[0, :5] = 0.0
    T = np.ascontiguousarray(m["t"][0][0])
    R = np.ascontiguousarray(m["rho"][0][0])
    va = np.full((nc, ny, nx), 5.0)
    vb = va.copy()
    O.load().orc_setvdrydep(nx, ny, nc, O.p(g["diam"]), O.p(zl), O.p(ldu), O.p(rl), O.p(znt), O.p(ust),
                            O.p(T), O.p(R), O.p(va))
    F.setvdrydep(nx, ny, nc, g["diam"], zl, ldu, rl, znt, ust, T, R, vb)
    assert np.all(va[0] == 5.0)  # > 100 um: untouched
    assert_close(vb, va, 1e-12, 0.0, "vdep")


def test_meteo_scale(st):
    s = st["s"]
    g, m = s.grid, s.met
    nx, ny, nz = g["nx"], g["ny"], g["nz"]
    arrs = {k: np.ascontiguousarray(m[k][0]) for k in ("u", "v", "w", "rho")}
    kh = np.ascontiguousarray(np.random.default_rng(1).uniform(100, 5000, (nz, ny, nx)))
    outs = []
    for impl in ("oracle", "gpu"):
        vx, vy, vz, rho = (arrs[k].copy() for k in ("u", "v", "w", "rho"))
        vz = np.ascontiguousarray(vz + 0.01)
        k1 = np.zeros_like(vx)
        dv = np.zeros_like(vx)
        if impl == "oracle":
            O.load().orc_meteo_scale(nx, ny, nz, 0, g["dX1"], g["dX2"], O.p(g["dz"]), O.p(g["Hm1"]),
                                     O.p(g["topg"]), O.p(vx), O.p(vy), O.p(vz), O.p(rho), O.p(kh), O.p(k1),
                                     O.p(dv))
        else:
            F.meteo_scale(nx, ny, nz, 0, g["dX1"], g["dX2"], g["dz"], g["Hm1"], g["topg"], vx, vy, vz, rho,
                          kh, k1, dv)
        outs.append((vx, vz, rho, k1, dv))
    for x, y, nm in zip(outs[1], outs[0], ("vx", "vz", "rho", "rkh1", "divu")):
        assert_same_bits(x, y, nm)
