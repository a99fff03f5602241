"""Error growth of the precision form (binary32 stencil, binary64 budgets,
accumulation and finddt) against the plain binary64 form over a long
forecast window.

Both forms run the same scenario through the Sources/Fall3d.f90 time loop
(f3d_run), in chunks of ``chunk_h`` simulated hours; f3d_run resumes where
the previous chunk ended, so the chunks are one uninterrupted run.  At each
chunk end the deposit maps (LOAD, COL_MASS, C_GRND of printres_nc) and the
concentration field are compared (relative L2 and Linf), and the mass-budget
logs (every 600 s, endstep.f90:51) give:

* ``closure``: |massvol + massdep + outmass - erumass| / erumass of each
  form: the scheme's own budget closure (cmass3d.f90:29-58, writim.f90:24-52),
  the same in both forms;
* ``massvol_rel_diff``: |massvol32 - massvol64| / massvol64;
* ``total_rel_diff``: |(massvol + massdep + outmass)32 - (...)64| / erumass:
  the mass the binary32 form gains or loses against the binary64 form.

Beside the measurement, ``storage_bound`` is the drift that rounding the
stored concentrations to binary32 alone would leave: unbiased rounding of
each cell's value (relative standard deviation ``SIGMA_U`` of the unit
roundoff) adds to the total mass M a random error of standard deviation
SIGMA_U * sqrt(sum_i m_i^2) per store, i.e. SIGMA_U * M / sqrt(N_eff) with
N_eff = M^2 / sum_i m_i^2 the effective number of cells carrying the mass;
independent stores over S steps add in quadrature.  N_eff is taken from the
binary64 field at each chunk end.

    python -m fall3d_gb300.accuracy [--hours 24] [--chunk-h 3] [--workload cfg1]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

import fall3d_gb300 as F
from fall3d_gb300 import _abi, synth

U32 = 2.0 ** -24  # unit roundoff of binary32 (round to nearest)
# standard deviation of the relative rounding error of a value whose
# significand f is log-uniform on [1, 2): the error is uniform on +-ulp/2
# (variance ulp^2/12) with ulp/x = 2^-23/f, and E[1/f^2] = 3/(8 ln 2), so
# SIGMA_U = 2^-23 * sqrt(1/(32 ln 2)) ~ 0.42 U32
SIGMA_U = 2.0 ** -23 * np.sqrt(1.0 / (32.0 * np.log(2.0)))


def _rel(a, b):
    d = np.asarray(a, np.float64) - b
    n, m = float(np.linalg.norm(b.ravel())), float(np.max(np.abs(b)))
    return {"rel_l2": float(np.linalg.norm(d.ravel())) / n if n > 0 else 0.0,
            "rel_linf": float(np.max(np.abs(d))) / m if m > 0 else 0.0}


def _n_eff(c, dz):
    """Effective number of cells carrying the mass of c (nc, nz+2, ny+2, nx+2)
    weighted by the layer thickness (the horizontal metric is nearly
    uniform on these grids)."""
    nz = c.shape[1] - 2
    m = c[:, 1:nz + 1, 1:-1, 1:-1] * np.asarray(dz[:nz])[None, :, None, None]
    s1, s2 = float(m.sum()), float(np.square(m).sum())
    return s1 * s1 / s2 if s2 > 0 else 0.0


def long_window(workload="cfg1", hours=24.0, chunk_h=3.0, seed=0):
    s = synth.make_scenario(workload, seed=seed, run_h=hours)
    g = s.grid
    nx, ny, nz, nc = g["nx"], g["ny"], g["nz"], g["nc"]
    met, src = _abi.make_met(s.met), _abi.make_src(s.src)
    g32, g64 = F.Context(s, F.PREC_FP32), F.Context(s, F.PREC_FP64)
    c32 = np.zeros((nc, nz + 2, ny + 2, nx + 2))
    c64 = np.zeros_like(c32)
    logs = {32: [], 64: []}
    rows, steps_done, var_sum = [], 0, 0.0
    wall = {32: 0.0, 64: 0.0}
    t_end = s.beg_time
    while t_end < s.end_time - 1e-9:
        t_end = min(s.end_time, t_end + chunk_h * 3600.0)
        for prec, ctx in ((32, g32), (64, g64)):
            t0 = time.perf_counter()
            logs[prec].append(ctx.run(end_time=t_end, met=met, src=src))
            wall[prec] += time.perf_counter() - t0
        st32, st64 = g32.state(), g64.state()
        o32, o64 = g32.outputs(), g64.outputs()
        g32.download_c(c32)
        g64.download_c(c64)
        n_eff = _n_eff(c64, g["dz"])
        steps = st64["iiter"] - steps_done
        steps_done = st64["iiter"]
        if n_eff > 0:
            var_sum += steps / n_eff
        l32 = {k: logs[32][-1][k][-1] for k in ("massvol", "massdep", "outmass", "erumass")}
        l64 = {k: logs[64][-1][k][-1] for k in ("massvol", "massdep", "outmass", "erumass")}
        tot32 = l32["massvol"] + l32["massdep"] + l32["outmass"]
        tot64 = l64["massvol"] + l64["massdep"] + l64["outmass"]
        eru = l64["erumass"]
        rows.append({
            "time_h": st64["time"] / 3600.0, "steps": st64["iiter"],
            "same_steps": st32["iiter"] == st64["iiter"] and st32["dt"] == st64["dt"],
            "load": _rel(o32["load"], o64["load"]), "col_mass": _rel(o32["col_mass"], o64["col_mass"]),
            "c_grnd": _rel(o32["c_grnd"], o64["c_grnd"]), "c": _rel(c32, c64),
            "massvol_rel_diff": abs(l32["massvol"] - l64["massvol"]) / abs(l64["massvol"]),
            "total_rel_diff": abs(tot32 - tot64) / eru,
            "closure_fp32": abs(tot32 - l32["erumass"]) / l32["erumass"],
            "closure_fp64": abs(tot64 - eru) / eru,
            "massvol_over_erumass": l64["massvol"] / eru,
            "n_eff": n_eff,
            "storage_bound_1sigma": SIGMA_U * np.sqrt(var_sum),
        })
    g32.close()
    g64.close()
    return {"workload": workload, "hours": hours, "chunk_h": chunk_h, "grid": [nx, ny, nz], "classes": nc,
            "wall_s": wall, "u32": U32, "sigma_u": SIGMA_U, "rows": rows}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="cfg1")
    ap.add_argument("--hours", type=float, default=24.0)
    ap.add_argument("--chunk-h", type=float, default=3.0)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()
    print(json.dumps(long_window(args.workload, args.hours, args.chunk_h, args.seed)))


if __name__ == "__main__":
    main()
