"""The large single-domain stress case: 1200x1000x80 at 0.01 deg, 30 classes
(including an aggregate class), wet deposition, Suzuki 25 km, 1e8 kg/s.

Runs ``steps`` steps of the precision form with CUDA-event timing of every
kernel (achieved HBM GB/s from the algorithmic bytes of each kernel), then
the same steps in the plain FP64 form, and reports the precision form's
relative L2 / Linf error of every 2-D output against it.

    python -m fall3d_gb300.stress [--steps 10] [--workload cfg4]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

import fall3d_gb300 as F
from fall3d_gb300 import synth


def _peak():
    import os

    p = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def run(workload="cfg4", steps=10, seed=0):
    t0 = time.perf_counter()
    s = synth.make_scenario(workload, seed=seed, max_snapshots=2)
    t_gen = time.perf_counter() - t0
    g = s.grid
    nx, ny, nz, nc = g["nx"], g["ny"], g["nz"], g["nc"]
    units = nx * ny * nz * nc
    peak, kind = _peak()

    def one(prec):
        ctx = F.Context(s, prec)
        ctx.source(0)
        t = time.perf_counter()
        ctx.meteo(0)
        ctx.sync()
        t_met = time.perf_counter() - t
        ctx.step(1)
        ctx.profile(True)
        ctx.step(steps)
        prof = ctx.profile_read()
        ctx.profile(False)
        b = ctx.budget()
        out = ctx.outputs()
        st = ctx.state()
        ctx.close()
        return prof, out, b, st, t_met

    prof32, out32, b32, st32, met32 = one(F.PREC_FP32)
    prof64, out64, b64, st64, met64 = one(F.PREC_FP64)

    # algorithmic bytes per cell-class of the step (12 + 28/nc binary32,
    # 24 + 56/nc binary64) over the step's kernels
    def rates(prof, S):
        res = {}
        tot = sum(v[1] for v in prof.values())
        for k, (n, ms) in prof.items():
            res[k] = {"ms_per_launch": ms / max(n, 1), "share": ms / tot if tot else 0.0}
        step_ms = tot / max(1, steps)
        bpc = 3 * S + 7 * S / nc
        res["_step"] = {"ms": step_ms, "cell_class_steps_per_s": units / (step_ms / 1e3),
                        "alg_bytes_per_cell_class": bpc,
                        "achieved_gbs": units * bpc / (step_ms / 1e3) / 1e9,
                        "frac_of_peak": units * bpc / (step_ms / 1e3) / 1e9 / peak}
        return res

    err = {}
    for k in ("load", "col_mass", "c_grnd"):
        d = out32[k] - out64[k]
        n64, m64 = float(np.linalg.norm(out64[k])), float(np.max(np.abs(out64[k])))
        err[k] = {"rel_l2": float(np.linalg.norm(d)) / n64 if n64 else 0.0,
                  "rel_linf": float(np.max(np.abs(d))) / m64 if m64 else 0.0}
    err["massvol"] = abs(b32["massvol"] - b64["massvol"]) / abs(b64["massvol"]) if b64["massvol"] else 0.0
    return {
        "workload": workload, "grid": [nx, ny, nz], "classes": nc, "steps": steps,
        "identical_step_sequence": st32["iiter"] == st64["iiter"] and st32["dt"] == st64["dt"],
        "fp32": rates(prof32, 4), "fp64": rates(prof64, 8),
        "meteo_update_s": {"fp32": met32, "fp64": met64}, "generation_s": t_gen,
        "peak_gbs": peak, "peak_source": kind, "fp32_vs_fp64": err,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="cfg4")
    ap.add_argument("--steps", type=int, default=10)
    args = ap.parse_args()
    print(json.dumps(run(args.workload, args.steps)))


if __name__ == "__main__":
    main()
