"""The input layer around the transport path: the reference's text input
files and the pre-processing utilities that write them, restated on the
host.

* ``.inp`` control file: ``read_inp`` / ``InpFile`` follow libMaster's
  get_input_rea/int/cha/npar (libMaster/get_input_rea.f90:1-118): the first
  line whose first word starts with the block name opens the block, the
  first following line whose first word starts with the keyword is the
  value line, words and numbers are split by blanks and '=' and numbers
  are decoded by libMaster/Decode.f90 (sdecode, decod1, stof, restated
  digit by digit so that every value has the reference's bits); ``FROM a
  TO b INCREMENT d`` expands to a, a+d, ... (get_input_rea.f90:54-72).
* ``.grn`` granulometry file: ``read_grn`` / ``write_grn``
  (libMaster/get_granulometry_value.f90:27-32, Utilities/SetTgsd/wrigrn.f90:16-21).
* ``.src`` source file: ``read_src`` / ``write_src`` (libMaster/
  get_source_value.f90:45-63, Utilities/SetSrc/wrisrc_mesh.f90:17-60),
  giving the f3d_src_series dict of the context (rates unscaled, as read)
  and the source heights zs.
* generators: ``setfrac`` (Utilities/SetTgsd/setfrac.f90: Gaussian and
  bi-Gaussian TGSD with the reference's trapezoidal normal CDF ``fer``),
  ``solvesuzuki`` (Utilities/SetSrc/solvesuzuki.f90) and ``getsrc``
  (Utilities/SetSrc/getsrc.f90: bilinear spreading over the four nodes
  around each column point, linear between the two model levels).
* ``setpsi`` / ``get_gama`` (Sources/setpsi.f90, called at
  Sources/readat.f90:248): the shape factor of each class for the settling
  model of the .inp, gama by the reference's bisection on the prolate
  ellipsoid's area.
* ``scenario_from_files``: a Scenario for fall3d_gb300.Context from an .inp,
  a .grn and a .src file (grid from the .inp GRID block as reagrd.f90 derives
  it from the DBS properties), with the meteorology of a DBS file
  (fall3d_gb300.dbs, libMaster/get_dbs_value_plane.f90 and reamet.f90) or
  synthetic (fall3d_gb300.synth).
"""
from __future__ import annotations

import math

import numpy as np

# ------------------------------------------------------------------ .inp


def _powi(x: float, n: int) -> float:
    """x**n for an integer n as gfortran evaluates it (__builtin_powi:
    binary powering, and 1/x**|n| for a negative n)."""
    if n < 0:
        return 1.0 / _powi(x, -n)
    r, b = 1.0, x
    while n:
        if n & 1:
            r = r * b
        n >>= 1
        if n:
            b = b * b
    return r


def stof(s: str) -> float:
    """libMaster/Decode.f90 stof: the digits of the integer part times
    10**(n-i), the fraction digits times 10**(-i), then the exponent."""
    ipos, n = 0, len(s)
    nsign = 1
    if s[ipos] == "+":
        ipos += 1
    elif s[ipos] == "-":
        nsign = -1
        ipos += 1
    vals = []
    while True:
        ch = s[ipos]
        if ch in "DEde.":
            break
        vals.append(int(ch) if ch.isdigit() else 0)
        ipos += 1
        if ipos == n:
            ipos -= 1
            break
    v = 0.0
    nv = len(vals)
    for i, d in enumerate(vals, start=1):
        v = v + d * _powi(10.0, nv - i)
    if s[ipos] == "." and ipos != n - 1:
        ipos += 1
        vals = []
        while True:
            ch = s[ipos]
            if ch in "DEde":
                break
            vals.append(int(ch) if ch.isdigit() else 0)
            ipos += 1
            if ipos == n:
                ipos -= 1
                break
        for i, d in enumerate(vals, start=1):
            v = v + d * _powi(10.0, -i)
    if s[ipos] in "DEde" and ipos != n - 1:
        ipos += 1
        esign = 1
        if s[ipos] == "+":
            ipos += 1
        elif s[ipos] == "-":
            esign = -1
            ipos += 1
        vals = []
        while True:
            vals.append(int(s[ipos]) if s[ipos].isdigit() else 0)
            ipos += 1
            if ipos == n:
                break
        expo = 0
        nv = len(vals)
        for i, d in enumerate(vals, start=1):
            expo = expo + d * 10 ** (nv - i)
        v = v * _powi(10.0, expo) if esign == 1 else v / _powi(10.0, expo)
    return nsign * v


def sdecode(card: str):
    """libMaster/Decode.f90 sdecode: (words, numbers) of a line; tokens are
    separated by blanks and '='; a token made only of digits, signs, 'D',
    'E', 'd', 'e' and '.' is a number (decod1)."""
    words, params = [], []
    for tok in card.replace("=", " ").split():
        if all(ch.isdigit() or ch in "+-DEde." for ch in tok):
            params.append(stof(tok))
        else:
            words.append(tok)
    return words, params


class InpFile:
    """The .inp control file, searched as libMaster's get_input_* do."""

    def __init__(self, path: str):
        with open(path, encoding="latin-1") as f:
            self.lines = [ln.rstrip("\n")[:256] for ln in f]

    def _line(self, block: str, key: str):
        i, n = 0, len(self.lines)
        while i < n:  # the block: first word starts with its name
            words, _ = sdecode(self.lines[i])
            i += 1
            if words and words[0].startswith(block):
                break
        else:
            raise KeyError(f"block {block} not found in the input file")
        while i < n:
            words, params = sdecode(self.lines[i])
            i += 1
            if words and words[0].startswith(key):
                return words, params
        raise KeyError(f"line {key} not found in the input file")

    def real(self, block: str, key: str, nval: int = 1):
        """get_input_rea (libMaster/get_input_rea.f90:21-79)."""
        words, params = self._line(block, key)
        if len(words) > 1 and words[1] in ("FROM", "from"):
            x0, xf = params[0], params[1]
            if x0 > xf:
                raise ValueError(f"error in line {key}")
            dx = min(xf - x0, params[2])
            npar = int((xf - x0) / dx) + 1
            params = [x0 + (i - 1) * dx for i in range(1, npar + 1)]
        if len(params) < nval:
            raise ValueError(f"too few parameters in line {key}")
        return params if nval == 0 else params[:nval]

    def integer(self, block: str, key: str, nval: int = 1):
        """get_input_int: the numbers of the line truncated to integers."""
        return [int(v) for v in self.real(block, key, nval)]

    def char(self, block: str, key: str, nval: int = 1):
        """get_input_cha: the words after the keyword."""
        words, _ = self._line(block, key)
        if len(words) - 1 < nval:
            raise ValueError(f"too few words in line {key}")
        return words[1:1 + nval]

    def npar(self, block: str, key: str) -> int:
        """get_input_npar: the count of numbers of the line."""
        return len(self.real(block, key, 0))


def read_inp(path: str) -> InpFile:
    return InpFile(path)


# ------------------------------------------------------------------ .grn


def write_grn(path: str, diam_mm, rhop, sphe, fc):
    """Utilities/SetTgsd/wrigrn.f90:16-21: nc, then f10.6 1x f8.1 1x f7.3 1x
    e16.9 per class (diameter in mm)."""
    with open(path, "w") as f:
        f.write(f"{len(diam_mm):5d}\n")
        for d, r, s, c in zip(diam_mm, rhop, sphe, fc):
            f.write(f"{d:10.6f} {r:8.1f} {s:7.3f} {_e16_9(c)}\n")


def read_grn(path: str) -> dict:
    """libMaster/get_granulometry_value.f90:27-32 (list-directed read of nc,
    then diameter (mm), density, sphericity and fraction per class)."""
    with open(path) as f:
        toks = f.read().split()
    try:  # a short or garbled file is the reader's error 101
        nc = int(toks[0])
        if nc < 0 or len(toks) < 1 + 4 * nc:
            raise IndexError
        rows = np.array([[_fortran_real(t) for t in toks[1 + 4 * i:5 + 4 * i]] for i in range(nc)]).reshape(nc, 4)
    except (IndexError, ValueError):
        raise ValueError(f"get_granulometry_value: error reading the granulometry file {path}") from None
    return dict(nc=nc, diam_mm=rows[:, 0], rhop=rows[:, 1], sphe=rows[:, 2], fc=rows[:, 3])


# ------------------------------------------------------------------ .src


def _e16_9(v: float) -> str:
    """Fortran e16.9: 0.ddddddddde+xx."""
    if v == 0.0:
        return "0.000000000E+00".rjust(16)
    m, e = f"{abs(v):.8e}".split("e")
    digits = m.replace(".", "")
    ex = int(e) + 1
    s = f"0.{digits[:9]}E{'+' if ex >= 0 else '-'}{abs(ex):02d}"
    return ("-" + s if v < 0 else s).rjust(16)


def _fortran_real(t: str) -> float:
    return float(t.replace("D", "E").replace("d", "e"))


def write_src(path: str, intervals, coord_sys="LON-LAT"):
    """Utilities/SetSrc/wrisrc_mesh.f90:31-60.  intervals: list of dicts
    with t1, t2, x, y, z, i, j, k (per source) and rates (nsou, nc)."""
    with open(path, "w") as f:
        for it in intervals:
            rates = np.asarray(it["rates"], float)
            ns = rates.shape[0]
            nc = rates.shape[1] if rates.ndim == 2 else 0
            f.write(f"{int(it['t1']):7d} {int(it['t2']):7d}\n")
            f.write(f"{ns:7d} {nc:7d}\n")
            f.write(f"{_e16_9(float(rates.sum()))}\n")
            for q in range(ns):
                if coord_sys == "LON-LAT":
                    xy = f" {it['x'][q]:11.6f} {it['y'][q]:11.6f}"
                else:
                    xy = f" {it['x'][q]:10.1f} {it['y'][q]:10.1f}"
                ijk = "".join(f" {int(v):5d}" for v in (it["i"][q], it["j"][q], it["k"][q]))
                vals = "".join(_e16_9(float(v)) + " " for v in rates[q])
                f.write(f"{xy}  {it['z'][q]:9.0f}  {ijk}  {vals}\n")


def read_src(path: str) -> dict:
    """The interval records of a .src file as libMaster's get_source_nsrc,
    get_source_coordinates and get_source_value read them (list-directed):
    itime1 itime2 / ns nc / MFR / ns lines of x y z i j k rates(nc).
    Returns the f3d_src_series dict (t1, t2, nsou, isrc, jsrc, ksrc,
    tmrat with rates (nsou_i, nc) column major per interval, as
    get_source_value stores them) plus zs, the source heights."""
    with open(path) as f:
        toks = f.read().split()
    pos = 0
    t1, t2, nsou, isrc, jsrc, ksrc, zs, tm = [], [], [], [], [], [], [], []
    nc_all = None
    tcur = 0
    while pos < len(toks):
        try:  # an incomplete or garbled interval record is the reader's error 101
            a, b = int(toks[pos]), int(toks[pos + 1])
            tcur = a
            ns, nc = int(toks[pos + 2]), int(toks[pos + 3])
            if ns < 0 or nc < 0 or pos + 5 + ns * (6 + nc) > len(toks):
                raise IndexError
            pos += 5  # MFR
            nc_all = nc if nc_all is None else nc_all
            rates = np.zeros((ns, nc))
            for q in range(ns):
                zs.append(_fortran_real(toks[pos + 2]))
                isrc.append(int(toks[pos + 3]))
                jsrc.append(int(toks[pos + 4]))
                ksrc.append(int(toks[pos + 5]))
                rates[q] = [_fortran_real(t) for t in toks[pos + 6:pos + 6 + nc]]
                pos += 6 + nc
        except (IndexError, ValueError):
            raise ValueError(f"get_source_value: error reading the source file at time {tcur:6d}") from None
        t1.append(a)
        t2.append(b)
        nsou.append(ns)
        tm.append(rates.T.reshape(-1))  # (ic-1)*ns + is
    return dict(t1=np.array(t1, np.int32), t2=np.array(t2, np.int32), nsou=np.array(nsou, np.int32),
                isrc=np.array(isrc, np.int32), jsrc=np.array(jsrc, np.int32), ksrc=np.array(ksrc, np.int32),
                tmrat=np.concatenate(tm) if tm else np.zeros(0), zs=np.array(zs), nc=nc_all or 0)


# ------------------------------------------------------------------ generators


def fer(x: float) -> float:
    """Utilities/SetTgsd/setfrac.f90:109-136: the standard normal CDF by the
    trapezoidal rule on 10000 steps of |x|/10000, divided by
    sqrt(8*atan(1.0)) with atan(1.0) in binary32 as the reference writes
    it (a default-real literal)."""
    fe = 0.0
    dt = abs(x) / 10000.0
    t1, t2 = 0.0, dt
    while True:
        fe = fe + 0.5 * (math.exp(-t1 * t1 / 2.0) + math.exp(-t2 * t2 / 2.0)) * dt
        t1 = t2
        t2 = t2 + dt
        if t2 >= abs(x):
            break
    fe = fe / math.sqrt(8.0 * float(np.arctan(np.float32(1.0))))
    return 0.5 + fe if x >= 0.0 else 0.5 - fe


def m0_fi_gaussian(fi, fimin, fimax, deltafi, fimean, fidisp):
    """Utilities/SetTgsd/setfrac.f90:64-102: the mass between fi-dfi/2 and
    fi+dfi/2, the end classes extended to +-infinity."""
    if fi == fimin:
        return fer((fimin + 0.5 * deltafi - fimean) / fidisp)
    if fi == fimax:
        return 1.0 - fer((fimax - 0.5 * deltafi - fimean) / fidisp)
    fc = fer((fi + 0.5 * deltafi - fimean) / fidisp)
    return fc - fer((fi - 0.5 * deltafi - fimean) / fidisp)


def setfrac(nc, fimin, fimax, rhomin, rhomax, sphemin, sphemax, fimean, fidisp):
    """Utilities/SetTgsd/setfrac.f90:17-45: diameters 2**-fi mm, density and
    sphericity linear in fi, fractions of one (GAUSSIAN) or two
    (BIGAUSSIAN: weights 0.98 and 0.02, binary32 literals) Gaussians."""
    fimean, fidisp = list(np.atleast_1d(fimean)), list(np.atleast_1d(fidisp))
    deltafi = (fimax - fimin) / (nc - 1)
    diam = np.zeros(nc)
    rhop = np.zeros(nc)
    sphe = np.zeros(nc)
    fc = np.zeros(nc)
    for ic in range(1, nc + 1):
        fi = fimin + (ic - 1) * deltafi
        diam[ic - 1] = 2.0 ** (-fi)
    for ic in range(1, nc + 1):
        fi = fimin + (ic - 1) * deltafi
        rhop[ic - 1] = (rhomax - rhomin) * (fi - fimin) / (fimax - fimin) + rhomin
        sphe[ic - 1] = (sphemax - sphemin) * (fi - fimin) / (fimax - fimin) + sphemin
    w98, w02 = float(np.float32(0.98)), float(np.float32(0.02))
    for ig in range(len(fimean)):
        for ic in range(1, nc + 1):
            fi = fimin + (ic - 1) * deltafi
            work = m0_fi_gaussian(fi, fimin, fimax, deltafi, fimean[ig], fidisp[ig])
            fc[ic - 1] = fc[ic - 1] + (w02 * work if ig > 0 else w98 * work)
    return dict(diam_mm=diam, rhop=rhop, sphe=sphe, fc=fc)


def solvesuzuki(ns, Hplume, Asuzu, Lsuzu, M0, fc, X0, Y0, Z0, dZ0):
    """Utilities/SetSrc/solvesuzuki.f90:19-46: column points z = is*H/ns above
    the vent, Suzuki weights normalised to M0, per class times fc.
    Returns (xplum, yplum, zplum (a.s.l.), mplum (nc, ns))."""
    S = np.zeros(ns)
    tot = 0.0
    deltaz = Hplume / ns
    zplum = np.zeros(ns)
    for is_ in range(1, ns + 1):
        z = is_ * deltaz
        S[is_ - 1] = ((1.0 - z / Hplume) * math.exp(Asuzu * (z / Hplume - 1.0))) ** Lsuzu
        zplum[is_ - 1] = Z0 + dZ0 + z
        tot = tot + S[is_ - 1]
    S = M0 * S / tot
    mplum = np.array([[fc[ic] * S[is_] for is_ in range(ns)] for ic in range(len(fc))])
    return np.full(ns, X0), np.full(ns, Y0), zplum, mplum


def getsrc(xplum, yplum, zplum, mplum, xorigr, yorigr, dx, dy, nx, ny, zmodel, topg, dZ0,
           terrain_following=True):
    """Utilities/SetSrc/getsrc.f90:16-107: each column point is spread over
    the four nodes of its cell with the bilinear shape functions
    (getshape, :112-136) and, at each node, linearly between the two model
    levels that bracket its height above that node's terrain.  Returns
    src (nc, nx, ny, nz) in the reference's index order."""
    nc, ns = mplum.shape
    nz = len(zmodel)
    src = np.zeros((nc, nx + 2, ny + 2, nz + 2))  # 1-based with room for ix+1, iz+1
    for is_ in range(ns):
        x, y, z = xplum[is_], yplum[is_], zplum[is_]
        ix = iy = None
        for i in range(1, nx + 1):
            if xorigr + (i - 1) * dx <= x <= xorigr + i * dx:
                ix = i
        if ix is None:
            raise ValueError("getsrc : source position not found in x")
        s = (x - (xorigr + (ix - 1) * dx)) / dx
        s = 2.0 * s - 1.0
        for i in range(1, ny + 1):
            if yorigr + (i - 1) * dy <= y < yorigr + i * dy:
                iy = i
        if iy is None:
            raise ValueError("getsrc : source position not found in y")
        t = (y - (yorigr + (iy - 1) * dy)) / dy
        t = 2.0 * t - 1.0
        sm, tm, sp, tp = 0.5 * (1.0 - s), 0.5 * (1.0 - t), 0.5 * (1.0 + s), 0.5 * (1.0 + t)
        shape = [sm * tm, sp * tm, sp * tp, sm * tp]
        nodes = [(ix, iy), (ix + 1, iy), (ix + 1, iy + 1), (ix, iy + 1)]
        iz, w = [0] * 4, [0.0] * 4
        for n_, (a, b) in enumerate(nodes):
            zp = topg[b - 1, a - 1] if terrain_following and a <= nx and b <= ny else 0.0
            k = 0
            while True:
                k += 1
                h = z - zp - dZ0
                if h < zmodel[0]:
                    w[n_] = 0.0
                    break
                if zmodel[k - 1] <= h < zmodel[k]:
                    w[n_] = (h - zmodel[k - 1]) / (zmodel[k] - zmodel[k - 1])
                    break
                if k == nz - 1:
                    raise ValueError("Source position not found in z")
            iz[n_] = k
        for ic in range(nc):
            m = mplum[ic, is_]
            for n_, (a, b) in enumerate(nodes):
                src[ic, a, b, iz[n_]] += (1.0 - w[n_]) * shape[n_] * m
                src[ic, a, b, iz[n_] + 1] += w[n_] * shape[n_] * m
    return src[:, 1:nx + 1, 1:ny + 1, 1:nz + 1]


def src_interval(src, t1, t2, xorigr, yorigr, dx, dy, zmodel):
    """wrisrc_mesh.f90:17-60: the nodes with a positive rate of any class,
    z fastest-outer order (iz, then iy, then ix), as one interval record."""
    nc, nx, ny, nz = src.shape
    rec = dict(t1=t1, t2=t2, x=[], y=[], z=[], i=[], j=[], k=[], rates=[])
    for iz in range(1, nz + 1):
        for iy in range(1, ny + 1):
            for ix in range(1, nx + 1):
                v = src[:, ix - 1, iy - 1, iz - 1]
                if np.any(v > 0.0):
                    rec["x"].append(xorigr + (ix - 1) * dx)
                    rec["y"].append(yorigr + (iy - 1) * dy)
                    rec["z"].append(zmodel[iz - 1])
                    rec["i"].append(ix)
                    rec["j"].append(iy)
                    rec["k"].append(iz)
                    rec["rates"].append(v.copy())
    rec["rates"] = np.array(rec["rates"]).reshape(-1, nc)
    return rec


# ------------------------------------------------------------------ scenario


def scenario_from_files(inp_path: str, grn_path: str, src_path: str, seed: int = 0, dbs_path: str = None,
                        **met_over):
    """A Scenario for fall3d_gb300.Context from the reference's input
    files: grid from the .inp GRID block (LON-LAT: LONMIN..LATMAX, NX, NY,
    ZLAYER_(M)), classes from the .grn file, sources from the .src file,
    run window from TIME_UTC; meteorology from the DBS file ``dbs_path``
    (fall3d_gb300.dbs.read_dbs on the grid's levels, Sources/reamet.f90), or
    synthetic (fall3d_gb300.synth) when none is given."""
    from fall3d_gb300 import synth

    inp = read_inp(inp_path)
    grn = read_grn(grn_path)
    srcd = read_src(src_path)
    nx, ny = inp.integer("GRID", "NX")[0], inp.integer("GRID", "NY")[0]
    zl = np.array(inp.real("GRID", "ZLAYER_(M)", 0))
    nz = len(zl)
    lonmin, lonmax = inp.real("GRID", "LONMIN")[0], inp.real("GRID", "LONMAX")[0]
    latmin, latmax = inp.real("GRID", "LATMIN")[0], inp.real("GRID", "LATMAX")[0]
    run_end_h = inp.real("TIME_UTC", "RUN_END_(HOURS_AFTER_00)")[0]
    beg_h = inp.real("TIME_UTC", "BEGIN_METEO_DATA_(HOURS_AFTER_00)")[0]
    nc = grn["nc"]
    if srcd["nc"] != nc:
        raise ValueError("the .src and .grn files disagree on the number of classes")
    over = dict(nx=nx, ny=ny, nz=nz, nc=nc, spacing=(lonmax - lonmin) / (nx - 1),
                lat0=0.5 * (latmin + latmax), ztop=float(zl[-1]),
                run_h=max(0.0, run_end_h - beg_h), H=0.5 * float(zl[-1]))  # synth's own column is replaced
    over.update(met_over)
    s = synth.make_scenario("small", seed=seed, **over)
    g = s.grid
    # reagrd.f90:149-182 from the .inp GRID block; the file's levels
    g["zlayer"] = zl
    dz = np.zeros(nz + 1)
    for k in range(1, nz):
        dz[k] = zl[k] - zl[k - 1]
    dz[0], dz[nz] = dz[1], dz[nz - 1]
    g["dz"] = dz
    g["diam"] = grn["diam_mm"] / 1e3
    g["rhop"] = grn["rhop"]
    g["sphe"] = np.minimum(grn["sphe"], 1.0)
    g["psi"] = setpsi(g["modv"], g["sphe"], g["diam"])  # Sources/readat.f90:248
    g["np"] = nc
    s.src = {k: srcd[k] for k in ("t1", "t2", "nsou", "isrc", "jsrc", "ksrc", "tmrat")}
    s.info["zs"] = list(srcd["zs"])
    s.info["fc"] = grn["fc"]
    if dbs_path is not None:
        from fall3d_gb300 import dbs

        met, warnings = dbs.read_dbs(dbs_path, zl, wetdep=bool(g["wetdep"]))
        if met["u"].shape[2:] != (ny, nx):
            raise ValueError("the DBS grid differs from the .inp GRID block")
        s.met = met
        s.info["dbs_warnings"] = warnings
    return s


def get_gama(diam, sphe):
    """Sources/setpsi.f90 get_gama: the axis ratio a/c of the prolate
    ellipsoid with the particle's volume and the area its sphericity gives,
    by bisection on [1e-3, 1] (at most 1000 halvings, until the area is
    within 1e-8), in the reference's operation order (diameter in m, scaled
    by 1e3; (0.5 d)**3 as (0.5 d)*((0.5 d)*(0.5 d)))."""
    d = diam * 1e3
    gmin, gmax = 1e-3, 1.0
    pi = 4.0 * math.atan(1.0)
    t = 0.5 * d
    vp = ((4.0 * pi) * (t * (t * t))) / 3.0
    ap = (math.pow(pi, 1.0 / 3.0) * math.pow(6.0 * vp, 2.0 / 3.0)) / sphe
    for it in range(1, 1001):
        gama = 0.5 * (gmin + gmax)
        e = math.acos(gama)
        ao = ((((0.5 * pi) * d) * d) * math.pow(gama, -(4.0 / 3.0))) * ((gama * gama) + (e / math.tan(e)))
        if ao < ap:
            gmax = gama
        else:
            gmin = gama
        if it > 1 and abs(ao - ap) < 1e-8:
            return gama
    raise RuntimeError("Subroutine get_gama: convergence not achieved")


def setpsi(modv, sphe, diam):
    """Sources/setpsi.f90 setpsi: the shape factor of each class for the
    settling model modv: 1 (Arastoopour) 1, 2 (Ganser) the sphericity,
    3 (Wilson) 0.5*(1 + 1/gama) for an oblate (gama >= 1) and gama for a
    prolate particle, 4 (Dellino) the sphericity over the circularity (1, or
    sqrt(gama) for a prolate particle), gama from get_gama."""
    sphe = np.asarray(sphe, dtype=np.float64)
    diam = np.asarray(diam, dtype=np.float64)
    if modv == 1:
        return np.ones_like(sphe)
    if modv == 2:
        return sphe.copy()
    out = np.zeros_like(sphe)
    for ic in range(len(sphe)):
        gama = get_gama(float(diam[ic]), float(sphe[ic]))
        if modv == 3:
            out[ic] = 0.5 * (1.0 + 1.0 / gama) if gama >= 1.0 else gama
        elif modv == 4:
            out[ic] = sphe[ic] / 1.0 if gama >= 1.0 else sphe[ic] / math.sqrt(gama)
    return out
