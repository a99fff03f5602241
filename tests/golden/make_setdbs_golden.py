"""Generates tests/golden/setdbs_abl.npz: the reference's own
Utilities/SetDbs/get_par_ABL.f90 (friction velocity and Monin-Obukhov
length of the DEBUG and the other met models of SetDbs) on fixed inputs.

    python tests/golden/make_setdbs_golden.py

oracle/ref_translate.py translates the routine into oracle/_ref/libsetdbs.so;
this script calls it on seeded inputs that cover the stable and unstable
branches, the wind floor (calm air), the thstar floor (equal potential
temperatures) and the DEBUG model's own columns, and stores inputs and
results; tests/test_dbs_cpu.py compares fall3d_gb300.dbs.get_par_abl with
them bit for bit.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def cases(seed=29):
    rng = np.random.default_rng(seed)
    n = 400
    z0 = np.ones(n)
    z1 = rng.uniform(20.0, 800.0, n)
    t0 = rng.uniform(250.0, 305.0, n)
    t1 = t0 + rng.uniform(-6.0, 6.0, n)
    p0 = rng.uniform(8.5e4, 1.03e5, n)
    p1 = p0 - rng.uniform(0.0, 8e3, n)
    u = rng.normal(0.0, 6.0, n)
    v = rng.normal(0.0, 6.0, n)
    # calm air (the 1e-4 wind floor), equal potential temperatures (the
    # thstar floor), the DEBUG model's columns (zlayer(2) of a few grids)
    u[:10] = 0.0
    v[:10] = 0.0
    t1[10:20] = t0[10:20]
    p1[10:20] = p0[10:20]
    for q, zz in enumerate((100.0, 250.0, 500.0, 1000.0)):
        i = 20 + q
        z1[i], t0[i], t1[i], p0[i], p1[i], u[i], v[i] = zz, 273.0, 273.0, 1e5, 1e5, 10.0, 0.0
    return dict(z0=z0, z1=z1, tz0=t0, tz1=t1, pz0=p0, pz1=p1, u=u, v=v)


def main():
    import ref_translate

    lib = C.CDLL(ref_translate.build_utility("setdbs"))
    f = lib.f90_get_par_abl
    f.restype = None
    c = cases()
    n = len(c["z0"])
    ust, rmo = np.zeros(n), np.zeros(n)
    for i in range(n):
        a = [C.c_double(float(c[k][i])) for k in ("z0", "z1", "tz0", "tz1", "pz0", "pz1", "u", "v")]
        o1, o2 = C.c_double(), C.c_double()
        f(*[C.byref(x) for x in a], C.byref(o1), C.byref(o2))
        ust[i], rmo[i] = o1.value, o2.value
    np.savez_compressed(os.path.join(HERE, "setdbs_abl.npz"), ustar=ust, rmonin=rmo, **c)
    print(f"{n} cases -> tests/golden/setdbs_abl.npz")


if __name__ == "__main__":
    main()
