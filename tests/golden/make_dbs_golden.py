"""Generates tests/golden/dbs_plane.npz: planes of a small meteorological
database (DBS) extracted by the reference's own libMaster/get_dbs_value_plane.f90.

    python tests/golden/make_dbs_golden.py

oracle/ref_translate.py translates that routine with its netCDF calls
replaced by accessors of an in-memory database (ref_dbs_set), so it runs on
the arrays stored here.  The database holds seeded binary32 fields on
non-uniform levels; the queries cover every record time, times between and
on the record boundaries, and heights below, on, between and above the
levels (on a level two intervals hold the height and the reference keeps the
last).  The fixture stores the database and, per query, the plane and the
end time the reference returns; tests/test_dbs_cpu.py writes the database
to a file with fall3d_gb300.dbs.write_dbs, reads it back through
fall3d_gb300.dbs.get_dbs_value_plane and compares bit for bit.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def database(seed=17):
    rng = np.random.default_rng(seed)
    nx, ny, nz, nt = 9, 7, 6, 3
    alt = np.array([0.0, 250.0, 700.0, 1500.0, 3100.0, 6000.0], np.float32)
    times = np.array([3600, 7200, 14400], np.int32)
    f32 = lambda a: np.asarray(a, np.float32)
    db = {"alt": alt, "times": times, "nx": nx, "ny": ny, "nz": nz, "nt": nt,
          "U": f32(rng.normal(8.0, 3.0, (nt, nz, ny, nx))),
          "RHO": f32(1.2 * np.exp(-alt[None, :, None, None] / 8000.0) + rng.normal(0, 1e-3, (nt, nz, ny, nx))),
          "PBLH": f32(rng.uniform(300.0, 1800.0, (nt, ny, nx))),
          "LDU": f32(rng.integers(1, 25, (ny, nx)))}
    return db


def queries(db):
    t = [int(x) for x in db["times"]]
    tq = t + [t[0] + 1, (t[0] + t[1]) // 2, t[1] - 1, t[2] - 1]
    a = [float(x) for x in db["alt"]]
    zq = a + [-5.0, 0.5 * (a[1] + a[2]), a[3] + 1e-3, 2345.678, a[-1] + 10.0, 9000.0]
    q = []
    for word in ("U", "RHO"):
        for tt in tq:
            for z in zq:
                q.append((word, tt, z))
    for tt in tq:
        q.append(("PBLH", tt, 0.0))
    q.append(("LDU", t[0], 0.0))
    return q


def main():
    import ref_translate

    lib = C.CDLL(ref_translate.build())
    db = database()
    nx, ny, nz, nt = db["nx"], db["ny"], db["nz"], db["nt"]
    rank = {"U": 2, "RHO": 2, "PBLH": 1, "LDU": 0}
    case = {"U": 2, "RHO": 2, "PBLH": 1, "LDU": 0}
    planes, ends, qs = [], [], queries(db)
    keep = []
    for word, tt, z in qs:
        data = np.ascontiguousarray(db[word])
        keep.append(data)
        lib.ref_dbs_set(nt, nz, nx, ny, rank[word], db["times"].ctypes.data_as(C.c_void_p),
                        db["alt"].ctypes.data_as(C.c_void_p), data.ctypes.data_as(C.c_void_p))
        var = np.zeros((ny, nx))
        endsec, istat = C.c_int(0), C.c_int(0)
        lib.f90_get_dbs_value_plane(C.byref(C.c_int(case[word])), C.byref(C.c_int(tt)), C.byref(C.c_double(z)),
                                    C.byref(C.c_int(nx)), C.byref(C.c_int(ny)), var.ctypes.data_as(C.c_void_p),
                                    C.byref(endsec), C.byref(istat))
        assert istat.value == 0, (word, tt, z)
        planes.append(var)
        ends.append(endsec.value)
    np.savez_compressed(os.path.join(HERE, "dbs_plane.npz"), alt=db["alt"], times=db["times"], U=db["U"],
                        RHO=db["RHO"], PBLH=db["PBLH"], LDU=db["LDU"],
                        q_word=np.array([w for w, _, _ in qs]), q_time=np.array([t for _, t, _ in qs], np.int32),
                        q_z=np.array([z for _, _, z in qs]), planes=np.array(planes), endsec=np.array(ends, np.int32))
    print(f"{len(qs)} planes -> tests/golden/dbs_plane.npz")


if __name__ == "__main__":
    main()
