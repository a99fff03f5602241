"""Generates tests/golden/setpsi.npz: the shape factors of the reference's
own Sources/setpsi.f90 (setpsi with get_gama) on fixed classes.

    python tests/golden/make_setpsi_golden.py

The routine is taken from the translated reference (oracle/_ref, built by
oracle/ref_translate.py) for the four settling models and seeded diameters
and sphericities; tests/test_inputs_cpu.py compares
fall3d_gb300.inputs.setpsi with it bit for bit.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def main():
    import ref_translate

    lib = C.CDLL(ref_translate.build())
    f = lib.f90_setpsi
    f.restype = None
    rng = np.random.default_rng(41)
    nc = 40
    diam = np.exp(rng.uniform(np.log(2e-6), np.log(4e-3), nc))
    sphe = rng.uniform(0.4, 1.0, nc)
    sphe[:3] = [1.0, 0.999, 0.5]
    out = {"diam": diam, "sphe": sphe}
    for modv in (1, 2, 3, 4):
        psi = np.zeros(nc)
        f(psi.ctypes.data_as(C.c_void_p), sphe.ctypes.data_as(C.c_void_p), diam.ctypes.data_as(C.c_void_p),
          C.byref(C.c_int(modv)), C.byref(C.c_int(nc)))
        out[f"psi{modv}"] = psi
    np.savez_compressed(os.path.join(HERE, "setpsi.npz"), **out)
    print(f"{nc} classes x 4 models -> tests/golden/setpsi.npz")


if __name__ == "__main__":
    main()
