"""Generates tests/golden/generators.npz: the reference's own pre-processing
generators run on fixed inputs.

    python tests/golden/make_generators_golden.py

oracle/ref_translate.py translates the utilities' Fortran into two
libraries of oracle/_ref/ (each utility has a Master module of its own):
SetTgsd (setfrac.f90: setfrac, M0_fi_gaussian, fer) and SetSrc
(solvesuzuki.f90; getsrc.f90: getsrc, getshape).  This script sets their
module variables through the libraries' symbols, calls the routines and
stores inputs and results; tests/test_generators_cpu.py compares
fall3d_gb300.inputs.setfrac / solvesuzuki / getsrc with them bit for bit.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# TGSD cases: (nc, fimin, fimax, rhomin, rhomax, sphemin, sphemax, fimean, fidisp)
TGSD = [(6, -1.0, 4.0, 1000.0, 2500.0, 0.9, 0.9, [1.5], [1.5]),
        (16, -2.0, 6.0, 800.0, 2700.0, 0.6, 0.95, [1.0, 4.5], [1.2, 0.8]),
        (9, 0.0, 8.0, 1200.0, 1200.0, 0.7, 1.0, [3.3], [2.1])]
# Suzuki column: (ns, Hplume, Asuzu, Lsuzu, M0, X0, Y0, Z0, dZ0)
SUZUKI = [(100, 8000.0, 4.0, 5.0, 1.0e6, 0.37, 0.41, 1500.0, 0.0),
          (50, 15000.0, 8.0, 1.5, 3.2e7, 0.52, 0.23, 900.0, 120.0)]
# getsrc grid: nx, ny, zmodel, xorigr, yorigr, dx, dy
GRID = dict(nx=20, ny=16, xorigr=0.0, yorigr=0.0, dx=0.05, dy=0.05,
            zmodel=np.array([0.0, 100.0, 300.0, 700.0, 1300.0, 2000.0, 3000.0, 4500.0, 6500.0, 9000.0,
                             12000.0, 16000.0, 21000.0]))


def arr(lib, name, ctype=C.c_double):
    return C.POINTER(ctype).in_dll(lib, name)


def set_alloc(lib, name, a, keep):
    """Points an allocatable module array of the translated library at ``a``
    (column-major values, lower bounds 1)."""
    a = np.asfortranarray(a, dtype=np.float64)
    keep.append(a)
    C.c_void_p.in_dll(lib, f"m_{name}").value = a.ctypes.data
    lb = (C.c_longlong * a.ndim).in_dll(lib, f"m_{name}_lb")
    ex = (C.c_longlong * a.ndim).in_dll(lib, f"m_{name}_ex")
    for d in range(a.ndim):
        lb[d], ex[d] = 1, a.shape[d]
    return a


def run_tgsd(lib, case):
    nc, fimin, fimax, rhomin, rhomax, smin, smax, fimean, fidisp = case
    C.c_int.in_dll(lib, "m_nc").value = nc
    C.c_int.in_dll(lib, "m_ng").value = len(fimean)
    for n, v in (("fimin", fimin), ("fimax", fimax), ("rhomin", rhomin), ("rhomax", rhomax),
                 ("sphemin", smin), ("sphemax", smax)):
        C.c_double.in_dll(lib, f"m_{n}").value = v
    fm = (C.c_double * 2).in_dll(lib, "m_fimean")
    fd = (C.c_double * 2).in_dll(lib, "m_fidisp")
    for i in range(len(fimean)):
        fm[i], fd[i] = fimean[i], fidisp[i]
    lib.f90_getmem()
    lib.f90_setfrac()
    out = {}
    for n in ("fc", "diam", "rhop", "sphe"):
        p = arr(lib, f"m_{n}")
        out[n] = np.array([p[i] for i in range(nc)])
    return out


def run_setsrc(lib, case, fc, topg, keep):
    ns, H, A, L, M0, X0, Y0, Z0, dZ0 = case
    nc = len(fc)
    ci = lambda n, v: setattr(C.c_int.in_dll(lib, f"m_{n}"), "value", int(v))
    cd = lambda n, v: setattr(C.c_double.in_dll(lib, f"m_{n}"), "value", float(v))
    ci("ns", ns)
    ci("nc", nc)
    for n, v in (("hplume", H), ("asuzu", A), ("lsuzu", L), ("m0", M0), ("x0", X0), ("y0", Y0), ("z0", Z0),
                 ("dz0", dZ0)):
        cd(n, v)
    set_alloc(lib, "fc", fc, keep)
    xp = set_alloc(lib, "xplum", np.zeros(ns), keep)
    yp = set_alloc(lib, "yplum", np.zeros(ns), keep)
    zp = set_alloc(lib, "zplum", np.zeros(ns), keep)
    mp = set_alloc(lib, "mplum", np.zeros((nc, ns)), keep)
    lib.f90_solvesuzuki()
    g = GRID
    nx, ny, nz = g["nx"], g["ny"], len(g["zmodel"])
    ci("nx", nx)
    ci("ny", ny)
    ci("nz", nz)
    for n in ("xorigr", "yorigr", "dx", "dy"):
        cd(n, g[n])
    set_alloc(lib, "zmodel", g["zmodel"], keep)
    set_alloc(lib, "topg", topg, keep)  # (nx+1, ny+1): the nodes ix+1, iy+1 of the last cells
    src = set_alloc(lib, "src", np.zeros((nc, nx + 1, ny + 1, nz + 1)), keep)
    lib.f90_getsrc()
    return dict(xplum=np.array(xp), yplum=np.array(yp), zplum=np.array(zp), mplum=np.array(mp),
                src=np.array(src))


def main():
    import ref_translate

    tg = C.CDLL(ref_translate.build_utility("settgsd"))
    ss = C.CDLL(ref_translate.build_utility("setsrc"))
    out, keep = {}, []
    for k, case in enumerate(TGSD):
        r = run_tgsd(tg, case)
        for n, v in r.items():
            out[f"tgsd{k}_{n}"] = v
    rng = np.random.default_rng(23)
    nx, ny = GRID["nx"], GRID["ny"]
    X, Y = np.meshgrid(np.arange(nx + 1) * GRID["dx"], np.arange(ny + 1) * GRID["dy"], indexing="ij")
    topg = 800.0 * np.exp(-((X - 0.45) ** 2 + (Y - 0.35) ** 2) / 0.05) + rng.uniform(0, 20, X.shape)
    out["topg"] = topg
    for k, case in enumerate(SUZUKI):
        fc = out[f"tgsd{k}_fc"]
        r = run_setsrc(ss, case, fc, topg, keep)
        for n, v in r.items():
            out[f"src{k}_{n}"] = v
    np.savez_compressed(os.path.join(HERE, "generators.npz"), **out)
    print(f"{len(out)} arrays -> tests/golden/generators.npz")


if __name__ == "__main__":
    main()
