"""Seeded synthetic scenarios for the transport step.

No public dataset is used by FALL3D 7.0 or by this project's workloads: every
input is generated here from a seed, with the shapes, sizes and value
distributions of the named workloads.  The generator restates

* the grid set-up of Sources/reagrd.f90:152-270 (dX1/dX2 from the lon-lat
  spacing, Hm1 = sin(colatitude), dz(0:nz) from zlayer with the two frame
  extensions of reagrd.f90:216-220);
* a standard atmosphere at z + topg as in the "standard" branch of
  Utilities/SetDbs/read_DEBUG_data.f90:45-66 (T, P, rho, TP = T (1e5/P)^0.285);
* the Gaussian total grain-size distribution of
  Utilities/SetTgsd/setfrac.f90:18-43 (phi grid, d = 2^-phi mm, linear
  density) and the PERCENTAGE aggregate class of
  Utilities/SetSrc/readgrn_erup.f90:148-161;
* the Suzuki column of Utilities/SetSrc/solvesuzuki.f90:25-45 distributed on
  the mesh as Utilities/SetSrc/getsrc.f90:23-106 does, with rates rounded to
  the e16.9 text precision of Utilities/SetSrc/wrisrc_mesh.f90:31-57.

DBS variables are binary32 in the reference
(Utilities/SetDbs/write_DBS_grid.f90:111-125), so every meteorological field
is rounded to float32 before it is widened to float64.

Arrays use numpy C order with the slowest index first, so a (nz, ny, nx)
array has the reference's (nx, ny, nz) Fortran layout in memory.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

PI = 3.14159265358979323846  # Sources/Numeric.f90:13
REARTH = 6356e3               # Sources/Numeric.f90:14

COORD_LONLAT, COORD_UTM = 0, 1
MODKV_CONSTANT, MODKV_SIMILARITY, MODKV_SURFACE = 0, 1, 2
MODKH_CONSTANT, MODKH_RAMS, MODKH_CMAQ = 0, 1, 2
MODV_ARASTOOPOUR, MODV_GANSER, MODV_WILSON, MODV_DELLINO = 1, 2, 3, 4


@dataclass
class Scenario:
    """One forecast: grid + classes (``grid``), meteorology and sources."""

    name: str
    seed: int
    grid: dict
    met: dict
    src: dict
    beg_time: float
    end_time: float
    info: dict = field(default_factory=dict)

    @property
    def cells(self) -> int:
        g = self.grid
        return g["nx"] * g["ny"] * g["nz"]

    @property
    def cell_classes(self) -> int:
        return self.cells * self.grid["nc"]


def _f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def standard_atmosphere(z):
    """ISA temperature (K), pressure (Pa), density (kg/m3) at altitude z (m)."""
    z = np.asarray(z, dtype=np.float64)
    g0, R, L, T0, P0 = 9.80665, 287.05, 0.0065, 288.15, 101325.0
    z11 = 11000.0
    T11 = T0 - L * z11
    P11 = P0 * (T11 / T0) ** (g0 / (R * L))
    zt = np.minimum(z, z11)
    T = np.where(z <= z11, T0 - L * zt, T11)
    P = np.where(z <= z11, P0 * (np.maximum(T, 1.0) / T0) ** (g0 / (R * L)),
                 P11 * np.exp(-g0 * (z - z11) / (R * T11)))
    rho = P / (R * T)
    return T, P, rho


def _smooth_noise(rng, shape2d, sigma_cells, amplitude):
    """Seeded Gaussian-filtered noise scaled to +/- amplitude (max abs)."""
    ny, nx = shape2d
    w = rng.standard_normal((ny, nx))
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.fftfreq(nx)[None, :]
    filt = np.exp(-2.0 * (math.pi * sigma_cells) ** 2 * (kx ** 2 + ky ** 2))
    f = np.real(np.fft.ifft2(np.fft.fft2(w) * filt))
    m = np.max(np.abs(f))
    return f * (amplitude / m) if m > 0 else f


def _spectral_noise(rng, shape2d, rms, slope=-5.0 / 3.0):
    """Seeded 2-D field with an isotropic k^slope energy spectrum, given rms."""
    ny, nx = shape2d
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.fftfreq(nx)[None, :]
    k = np.sqrt(kx ** 2 + ky ** 2)
    k[0, 0] = 1.0
    # energy E(k) ~ k^slope in 2-D -> amplitude ~ sqrt(E(k)/k)
    amp = np.sqrt(k ** slope / k)
    amp[0, 0] = 0.0
    phase = rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))
    f = np.real(np.fft.ifft2(amp * phase))
    s = np.std(f)
    return f * (rms / s) if s > 0 else f


def make_classes(nc, phimin, phimax, rho_coarse=2500.0, rho_fine=1000.0,
                 sphe=0.9, mu=1.5, sigma=1.5, aggregate=None):
    """TGSD of Utilities/SetTgsd/setfrac.f90:18-43: phi grid, d = 2^-phi mm,
    density linear in phi from rho_coarse (phimin) to rho_fine (phimax),
    Gaussian mass fractions in phi.  With ``aggregate`` = (diam_mm, rho,
    fraction), the last class is an aggregate receiving ``fraction`` of the
    mass of every finer class (readgrn_erup.f90:148-161, PERCENTAGE)."""
    npart = nc - (1 if aggregate else 0)
    phis = np.linspace(phimin, phimax, npart) if npart > 1 else np.array([phimin], float)
    dphi = (phimax - phimin) / (npart - 1) if npart > 1 else 1.0
    diam_mm = 2.0 ** (-phis)
    t = (phis - phimin) / (phimax - phimin) if phimax > phimin else np.zeros_like(phis)
    rhop = rho_coarse + (rho_fine - rho_coarse) * t
    cdf = lambda x: 0.5 * (1.0 + math.erf((x - mu) / (sigma * math.sqrt(2.0))))
    fc = np.array([cdf(p + 0.5 * dphi) - cdf(p - 0.5 * dphi) for p in phis])
    fc[0] += cdf(phis[0] - 0.5 * dphi)
    fc[-1] += 1.0 - cdf(phis[-1] + 0.5 * dphi)
    fc = fc / fc.sum()
    names = [f"class-{i + 1:02d}" for i in range(npart)]
    sph = np.full(npart, sphe)
    if aggregate:
        d_ag, rho_ag, frac = aggregate
        fca = 0.0
        for ic in range(npart):
            if d_ag > diam_mm[ic]:
                fca += frac * fc[ic]
                fc[ic] = (1.0 - frac) * fc[ic]
        diam_mm = np.append(diam_mm, d_ag)
        rhop = np.append(rhop, rho_ag)
        sph = np.append(sph, sphe)
        fc = np.append(fc, fca)
        names.append("aggregate")
    # .grn text precision (readgrn_erup.f90:194-198): f10.6 mm, f8.1, f7.3
    diam_mm = np.array([float(f"{v:.6f}") for v in diam_mm])
    rhop = np.array([float(f"{v:.1f}") for v in rhop])
    sph = np.minimum(np.array([float(f"{v:.3f}") for v in sph]), 1.0)  # reagrn.f90:57
    return dict(diam=diam_mm / 1e3, rhop=rhop, sphe=sph, fc=fc, names=names)


def setpsi(modv, sphe, diam):
    """Shape factor psi of Sources/setpsi.f90:27-58, as the reference derives
    it from the classes (Sources/readat.f90:248): 1 (ARASTOOPOUR), the
    sphericity (GANSER), and from get_gama's axis ratio for WILSON and
    DELLINO (fall3d_gb300.inputs.setpsi)."""
    from fall3d_gb300 import inputs

    return inputs.setpsi(modv, np.asarray(sphe, dtype=np.float64), np.asarray(diam, dtype=np.float64))


def suzuki_column(ns, H, A, lam, M0, fc):
    """Utilities/SetSrc/solvesuzuki.f90:25-45: heights above the vent and the
    mass rate of each class at each of the ns column points."""
    deltaz = H / ns
    z = np.arange(1, ns + 1) * deltaz
    S = ((1.0 - z / H) * np.exp(A * (z / H - 1.0))) ** lam
    S = M0 * S / S.sum()
    return z, np.outer(S, fc)  # (ns, nc)


def distribute_column(zrel, mplum, zlayer, nz):
    """Vertical part of Utilities/SetSrc/getsrc.f90:71-100 for a vent on a
    grid node (all horizontal weight on that node): each column point is
    split linearly between the two model levels that bracket it."""
    src = np.zeros((nz, mplum.shape[1]))
    for is_, z in enumerate(zrel):
        if z < zlayer[0]:
            iz, w = 0, 0.0
        else:
            iz = None
            for k in range(nz - 1):
                if zlayer[k] <= z < zlayer[k + 1]:
                    iz = k
                    break
            if iz is None:
                raise ValueError("source position not found in z")
            w = (z - zlayer[iz]) / (zlayer[iz + 1] - zlayer[iz])
        src[iz] += (1.0 - w) * mplum[is_]
        src[iz + 1] += w * mplum[is_]
    return src


def _grid(nx, ny, nz, spacing, lat0, ztop, coord=COORD_LONLAT, lon0=14.0):
    """Sources/reagrd.f90:152-270 for a regular lon-lat (or UTM) grid."""
    if coord == COORD_LONLAT:
        lonmin = lon0
        latmin = lat0 - 0.5 * spacing * (ny - 1)
        lonmax = lonmin + spacing * (nx - 1)
        latmax = latmin + spacing * (ny - 1)
        dx = (lonmax - lonmin) / (nx - 1)
        dy = (latmax - latmin) / (ny - 1)
        dX1 = REARTH * (dx * PI / 180.0)
        dX2 = REARTH * (dy * PI / 180.0)
        Hm1 = np.empty((ny, nx))
        for j in range(ny):
            lat = latmin + j * dy
            colat = (90.0 - lat) * PI / 180.0
            Hm1[j, :] = math.sin(colat)
        xs = lonmin + np.arange(nx) * dx
        ys = latmin + np.arange(ny) * dy
    else:
        dx = dy = spacing
        dX1, dX2 = dx, dy
        Hm1 = np.ones((ny, nx))
        xs = np.arange(nx) * dx
        ys = np.arange(ny) * dy
    zlayer = _f32(np.linspace(0.0, ztop, nz))
    dz = np.zeros(nz + 1)
    for k in range(1, nz):
        dz[k] = zlayer[k] - zlayer[k - 1]
    dz[0] = dz[1]
    dz[nz] = dz[nz - 1]
    return dict(dx=dx, dy=dy, dX1=dX1, dX2=dX2, Hm1=Hm1, zlayer=zlayer, dz=dz, xs=xs, ys=ys)


def make_scenario(name="cfg0", seed=0, **over) -> Scenario:
    """Build a named workload.  ``over`` overrides any parameter below.

    cfg0   80x80x25 at 0.05 deg, 6 classes phi -1..4, Suzuki 8 km, MER 1e6 kg/s
           for 1 h, run 3 h, hourly identical snapshots (the CPU-sized case).
    cfg1   400x300x50 at 0.02 deg, 16 classes phi -2..6, k^-5/3 wind
           perturbation (5 m/s rms), precipitation band 0-5 mm/h, wet
           deposition on, Suzuki 15 km, MER 1e7 kg/s for 3 h, run 24 h,
           snapshots every 30 min interpolated between two base states 1 h
           apart.
    cfg4   1200x1000x80 at 0.01 deg, 30 classes incl. a 20% aggregate class,
           6-hourly snapshots, Suzuki 25 km, MER 1e8 kg/s for 6 h, run 48 h.
    tiny / small   reduced cfg0-like grids for tests.
    """
    presets = {
        "tiny": dict(nx=12, ny=10, nz=8, nc=3, phimin=0.0, phimax=4.0, spacing=0.05, ztop=6000.0,
                     H=4000.0, M0=1e6, erupt_h=1.0, run_h=0.5, met_dt_h=1.0, pert=2.0,
                     spectral=False, wetdep=False, hill=800.0),
        "small": dict(nx=32, ny=28, nz=14, nc=4, phimin=-1.0, phimax=4.0, spacing=0.05, ztop=10000.0,
                      H=8000.0, M0=1e6, erupt_h=1.0, run_h=1.0, met_dt_h=0.5, pert=2.0,
                      spectral=False, wetdep=False, hill=1500.0),
        "cfg0": dict(nx=80, ny=80, nz=25, nc=6, phimin=-1.0, phimax=4.0, spacing=0.05, ztop=10000.0,
                     H=8000.0, M0=1e6, erupt_h=1.0, run_h=3.0, met_dt_h=1.0, pert=2.0,
                     spectral=False, wetdep=False, hill=1500.0),
        "cfg1": dict(nx=400, ny=300, nz=50, nc=16, phimin=-2.0, phimax=6.0, spacing=0.02, ztop=20000.0,
                     H=15000.0, M0=1e7, erupt_h=3.0, run_h=24.0, met_dt_h=0.5, pert=5.0,
                     spectral=True, wetdep=True, hill=1500.0),
        "cfg4": dict(nx=1200, ny=1000, nz=80, nc=30, phimin=-2.0, phimax=7.0, spacing=0.01, ztop=30000.0,
                     H=25000.0, M0=1e8, erupt_h=6.0, run_h=48.0, met_dt_h=6.0, pert=5.0,
                     spectral=True, wetdep=True, hill=1500.0, aggregate=(0.2, 1000.0, 0.2)),
    }
    if name not in presets:
        raise ValueError(f"unknown workload {name!r}")
    p = dict(presets[name])
    p.update(dict(lat0=37.5, A=4.0, lam=5.0, ns=100, modkv=MODKV_SIMILARITY, modkh=MODKH_RAMS,
                  modv=MODV_GANSER, coord=COORD_LONLAT, Csh=0.2275, rkh0=0.0, rkv0=0.0,
                  safety=0.9, sphe=0.9, mu=1.5, sigma=1.5, ust=0.3, pblh=1000.0, rmol=1.0 / 500.0,
                  znt=0.1, vy0=3.0, u10=10.0, max_snapshots=None, aggregate=p.get("aggregate")))
    p.update(over)
    rng = np.random.default_rng(seed)
    nx, ny, nz = p["nx"], p["ny"], p["nz"]
    g = _grid(nx, ny, nz, p["spacing"], p["lat0"], p["ztop"], p["coord"])
    iv, jv = (nx - 1) // 2, (ny - 1) // 2  # vent on the centre node (0-based)
    # Gaussian hill centred on the vent (sigma = 0.5 deg, or 10 cells on small grids)
    sig = 0.5 if p["coord"] == COORD_LONLAT else 10.0 * p["spacing"]
    sig = min(sig, 0.25 * p["spacing"] * min(nx, ny))
    X, Y = np.meshgrid(g["xs"] - g["xs"][iv], g["ys"] - g["ys"][jv])
    topg = _f32(p["hill"] * np.exp(-(X ** 2 + Y ** 2) / (2.0 * sig ** 2)))
    cls = make_classes(p["nc"], p["phimin"], p["phimax"], sphe=p["sphe"], mu=p["mu"],
                       sigma=p["sigma"], aggregate=p["aggregate"])
    nc = len(cls["diam"])
    psi = p.get("psi")
    if psi is None:
        psi = setpsi(p["modv"], cls["sphe"], cls["diam"])

    # --- meteorology -------------------------------------------------
    run_s = int(round(p["run_h"] * 3600))
    met_dt = int(round(p["met_dt_h"] * 3600))
    times = list(range(0, run_s + met_dt, met_dt))
    if p["max_snapshots"]:
        times = times[: p["max_snapshots"]]
    nt = len(times)
    zl = g["zlayer"]
    zabs = zl[:, None, None] + topg[None, :, :]
    T, P, RHO = standard_atmosphere(zabs)
    TP = T * (1e5 / P) ** 0.285
    prof = p["u10"] * (np.maximum(zl, 1.0) / 1000.0) ** 0.25  # terrain-following level height

    def wind_state(seed_off):
        r = np.random.default_rng(seed * 1000 + seed_off)
        if p["spectral"]:
            du = _spectral_noise(r, (ny, nx), p["pert"])
            dv = _spectral_noise(r, (ny, nx), p["pert"])
        else:
            du = _smooth_noise(r, (ny, nx), max(2.0, 0.1 * min(nx, ny)), p["pert"])
            dv = np.zeros((ny, nx))
        U = prof[:, None, None] + du[None] * (0.5 + 0.5 * zl[:, None, None] / zl[-1])
        V = p["vy0"] + dv[None] * np.ones((nz, 1, 1))
        return U, V

    UA, VA = wind_state(1)
    if p["spectral"]:
        UB, VB = wind_state(2)
    else:
        UB, VB = UA, VA
    shape3 = (nt, nz, ny, nx)
    met = {k: np.empty(shape3) for k in ("u", "v", "w", "t", "tp", "rho")}
    met2 = {k: np.empty((nt, ny, nx)) for k in ("ust", "pblh", "rmol", "znt", "prate")}
    X2, Y2 = np.meshgrid(np.arange(nx), np.arange(ny))
    for it, tt in enumerate(times):
        ph = (tt / 3600.0) % 2.0
        wgt = ph if ph <= 1.0 else 2.0 - ph  # triangle between the two base states
        met["u"][it] = _f32(UA + (UB - UA) * wgt)
        met["v"][it] = _f32(VA + (VB - VA) * wgt)
        met["w"][it] = 0.0
        met["t"][it] = _f32(T)
        met["tp"][it] = _f32(TP)
        met["rho"][it] = _f32(RHO)
        met2["ust"][it] = _f32(np.full((ny, nx), p["ust"]))
        met2["pblh"][it] = _f32(np.full((ny, nx), p["pblh"]))
        met2["rmol"][it] = _f32(np.full((ny, nx), p["rmol"]))
        met2["znt"][it] = _f32(np.full((ny, nx), p["znt"]))
        if p["wetdep"]:
            # a band of 0..5 mm/h drifting across the domain, stored in mm/s
            cx = (0.3 + 0.4 * wgt) * nx
            band = 5.0 * np.exp(-((X2 - cx) / (0.08 * nx)) ** 2)
            met2["prate"][it] = _f32(band / 3600.0)
        else:
            met2["prate"][it] = 0.0
    met.update(met2)
    met["times"] = np.array(times, dtype=np.int32)
    met["time_lag"] = 0.0
    met["ldu"] = _f32(np.full((ny, nx), -99.0))

    # --- source ------------------------------------------------------
    zrel, mplum = suzuki_column(p["ns"], p["H"], p["A"], p["lam"], p["M0"], cls["fc"])
    col = distribute_column(zrel, mplum, zl, nz)  # (nz, nc)
    ks = [k for k in range(nz) if np.any(col[k] > 0.0)]
    nsou = len(ks)
    tm = np.array([[float(f"{col[k, ic]:.9e}") for ic in range(nc)] for k in ks])
    erupt_s = int(round(p["erupt_h"] * 3600))
    t_end_src = max(run_s, erupt_s) + 10 * 86400
    src = dict(t1=np.array([0, erupt_s], np.int32), t2=np.array([erupt_s, t_end_src], np.int32),
               nsou=np.array([nsou, 0], np.int32),
               isrc=np.full(nsou, iv + 1, np.int32), jsrc=np.full(nsou, jv + 1, np.int32),
               ksrc=np.array([k + 1 for k in ks], np.int32),
               tmrat=np.asfortranarray(tm).T.reshape(-1).copy())  # (nsou,nc) column major

    grid = dict(nx=nx, ny=ny, nz=nz, nc=nc, np=nc, coord_sys=p["coord"], modkv=p["modkv"],
                modkh=p["modkh"], modv=p["modv"], wetdep=int(p["wetdep"]),
                aggregate=int(bool(p["aggregate"])), dX1=g["dX1"], dX2=g["dX2"], dx=g["dx"],
                dy=g["dy"], rkh0=p["rkh0"], rkv0=p["rkv0"], Csh=p["Csh"],
                safety_factor=p["safety"], vset_factor=1.0, dz=g["dz"], zlayer=zl,
                Hm1=g["Hm1"], topg=topg, diam=cls["diam"], rhop=cls["rhop"], psi=np.asarray(psi, float),
                sphe=cls["sphe"])
    info = dict(params=p, classes=cls["names"], fc=cls["fc"], vent=(iv + 1, jv + 1),
                origin=(float(g["xs"][0]), float(g["ys"][0])),
                vent_xy=(float(g["xs"][iv]), float(g["ys"][jv])),
                zs=[float(zl[k]) for k in ks])
    return Scenario(name=name, seed=seed, grid=grid, met=met, src=src, beg_time=0.0,
                    end_time=float(run_s), info=info)


def gravity_current(scen: Scenario, c_flow_rate=430.0, lambda_grav=0.2, k_entrain=0.1,
                    brunt_vaisala=0.02) -> dict:
    """Parameters of the GRAVITY_CURRENT block (Sources/readat.f90:150-213)
    for a scenario: the centre on the vent, the grid origin (reagrd.f90:152)
    and the top of the source column (maxval(zs), the source points'
    heights)."""
    return dict(c_flow_rate=c_flow_rate, lambda_grav=lambda_grav, k_entrain=k_entrain,
                brunt_vaisala=brunt_vaisala, center_x=scen.info["vent_xy"][0],
                center_y=scen.info["vent_xy"][1], xorigr=scen.info["origin"][0],
                yorigr=scen.info["origin"][1], h_tot=max(scen.info["zs"]) if scen.info["zs"] else 0.0,
                beg_time=scen.beg_time)


def add_gas_class(scen: Scenario, rate_fraction=0.05) -> Scenario:
    """Appends one gas species (class np+1, the first gas, which the
    aggregation model reads as magmatic water, agrsrc.f90:262-266) emitted
    with the source at ``rate_fraction`` of each source point's particle
    rate."""
    g = scen.grid
    nc, ns = g["nc"], int(np.sum(scen.src["nsou"]))
    g["np"] = g.get("np", nc)
    for k, v in (("diam", 1e-6), ("rhop", 1.0), ("sphe", 1.0), ("psi", 1.0)):
        g[k] = np.append(np.asarray(g[k], float), v)
    tm = np.asarray(scen.src["tmrat"], float)
    rows = []  # per interval: (nsou_i, nc) column major
    off = 0
    for n in scen.src["nsou"]:
        n = int(n)
        blk = tm[off * nc:(off + n) * nc].reshape(nc, n) if n else np.zeros((nc, 0))
        gas = np.array([float(f"{v:.9e}") for v in rate_fraction * blk.sum(axis=0)])
        rows.append(np.vstack([blk, gas[None, :]]).reshape(-1))
        off += n
    scen.src["tmrat"] = np.concatenate(rows) if rows else tm
    g["nc"] = nc + 1
    scen.info["fc"] = np.append(np.asarray(scen.info["fc"], float), 0.0)
    assert off == ns
    return scen


def aggregation_inputs(scen: Scenario, Df=2.8, ndtagr=2, rh_band=(2000.0, 5000.0)) -> dict:
    """Inputs of the aggregation model for a scenario (AGGREGATION block of
    readat.f90:350-440, the DBS variables QV and P, and the plume
    temperature file read by settemplume, source.f90:89-149):

    * fc: the .grn mass fractions; Df, ndtagr;
    * qv, p (per met snapshot): ISA pressure at the levels' heights above sea
      level and a specific humidity at 120% of saturation (over water, the
      formula of agrsrc.f90:402) in the height band rh_band, 30% elsewhere;
    * plume (per source interval): the source column's cells with
      temperatures from 500 K at the vent down to 230 K at the top (vapour,
      water and ice phases) and a water rate."""
    g = scen.grid
    nx, ny, nz = g["nx"], g["ny"], g["nz"]
    zl = np.asarray(g["zlayer"])
    zabs = zl[:, None, None] + np.asarray(g["topg"])[None]
    T, P, _ = standard_atmosphere(zabs)
    ew = 100.0 * 6.112 * np.exp(17.67 * (T - 273.16) / (T - 273.16 + 243.5))
    ws = 0.622 * ew / np.maximum(P - ew, 1.0)
    rh = np.where((zl[:, None, None] >= rh_band[0]) & (zl[:, None, None] <= rh_band[1]), 1.2, 0.3)
    w = rh * ws
    qv = _f32(w / (1.0 + w))
    nt = len(scen.met["times"])
    iv, jv = scen.info["vent"]
    plume = []
    for n in scen.src["nsou"]:
        if int(n) == 0:
            plume.append(dict(ix=np.zeros(0, np.int32), iy=np.zeros(0, np.int32), iz=np.zeros(0, np.int32),
                              t=np.zeros(0), w=np.zeros(0)))
            continue
        ks = np.array([int(k) for k in scen.src["ksrc"][:int(n)]], np.int32)
        frac = (ks - ks.min()) / max(1, ks.max() - ks.min())
        plume.append(dict(ix=np.full(len(ks), iv, np.int32), iy=np.full(len(ks), jv, np.int32), iz=ks,
                          t=_f32(500.0 - 270.0 * frac), w=_f32(1e3 * (1.0 - frac))))
    return dict(Df=float(Df), ndtagr=int(ndtagr), fc=np.asarray(scen.info["fc"][:g["np"]], float),
                qv=np.repeat(qv[None], nt, axis=0), p=np.repeat(_f32(P)[None], nt, axis=0), plume=plume)


def ensemble_member(seed: int, run_h: float = 12.0, max_snapshots=None, met_dt_h: float = 1.0) -> Scenario:
    """One member of the batched ensemble: nx, ny ~ U[64,320], nz ~ U[20,60],
    spacing 0.02-0.05 deg, 4-20 classes over phi -2..6, column 3-20 km, MER
    log-uniform 1e4-1e8 kg/s for 1-6 h, seeded wind perturbation; met
    snapshots every met_dt_h hours."""
    r = np.random.default_rng(10_000 + seed)
    nx = int(r.integers(64, 321))
    ny = int(r.integers(64, 321))
    nz = int(r.integers(20, 61))
    nc = int(r.integers(4, 21))
    spacing = float(np.round(r.uniform(0.02, 0.05), 4))
    H = float(r.uniform(3000.0, 20000.0))
    M0 = float(10 ** r.uniform(4.0, 8.0))
    erupt_h = float(r.uniform(1.0, 6.0))
    ztop = float(max(10000.0, 1.3 * H))
    return make_scenario("cfg0", seed=seed, nx=nx, ny=ny, nz=nz, nc=nc, phimin=-2.0, phimax=6.0,
                         spacing=spacing, ztop=ztop, H=H, M0=M0, erupt_h=erupt_h, run_h=run_h,
                         met_dt_h=met_dt_h, pert=3.0, spectral=False, max_snapshots=max_snapshots)
