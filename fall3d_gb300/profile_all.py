"""Launches every kernel of the library at least once, on the workloads the
per-kernel DRAM table is measured on:

* the 400x300x50 grid with 16 classes (precipitation band, wet deposition on)
  in both forms: one meteo update (the coefficient chain, finddt, the
  binary32 copies and halo-layout fields), two steps of every step path
  (per-routine binary64 sweeps, per-routine binary32 sweeps, the fused step
  of every tile shape), the budgets, every output variable and a flight
  level cut;
* a run of the precision form across a DBS boundary through f3d_run (the
  look-ahead meteo update: the settling chain beside the step kernel);
* a batch of four ensemble members (setsrc/cmass2d of every member, the
  persistent step kernel, the batch-step counters);
* a 64x56x20 grid with the gravity current and with aggregation in transport
  (addradialwind, divcorr, agrpar, agrsrc), whose fields fit in L2.

    python -m fall3d_gb300.profile_all [--workload cfg1]

It prints the kernel launch count; run it under a profiler to read each
kernel's duration and DRAM bytes.
"""
from __future__ import annotations

import argparse

import numpy as np

import fall3d_gb300 as F
from fall3d_gb300 import synth


def _context_kernels(s, prec, steps=2):
    g = F.Context(s, prec)
    g.source(0)
    g.meteo(0)
    if prec == F.PREC_FP32:
        for fused, tile in ((0, 0), (1, 0), (1, 1), (1, 2), (1, 3)):
            g.set_option(F.OPT_FUSED, fused)
            g.set_option(F.OPT_TILE, tile)
            g.step(steps)
        g.set_option(F.OPT_FUSED, 1)
        g.set_option(F.OPT_TILE, 3)
    else:
        g.step(steps)
    g.budget()
    g.count_nonfinite()
    for var, index in ((F.OUT_LOAD, 0), (F.OUT_WET, 0), (F.OUT_THICK, 0), (F.OUT_COL_MASS, 0),
                       (F.OUT_PM_COL, 10), (F.OUT_C_GRND, 0), (F.OUT_PM_GRND, 10), (F.OUT_AOT05, 0),
                       (F.OUT_CON, 0)):
        g.output(var, index)
    g.output(F.OUT_CON, 0, asl=True)
    zl = np.asarray(s.grid["zlayer"], dtype=np.float64)
    p = np.ascontiguousarray(np.broadcast_to((1.0e5 * np.exp(-zl / 8000.0))[:, None, None],
                                             (s.grid["nz"], s.grid["ny"], s.grid["nx"])))
    g.output_fl(100, p)  # FL100 through the isothermal-atmosphere pressure of the levels
    g.sync()
    g.close()


def run(workload="cfg1"):
    n0 = F.kernel_launches()
    s = synth.make_scenario(workload, seed=0, max_snapshots=2)
    _context_kernels(s, F.PREC_FP64)
    _context_kernels(s, F.PREC_FP32)
    # f3d_run across a DBS boundary: the look-ahead update of the second
    # snapshot (k_chain_beside, and the 112-register step kernel for steps
    # launched while it runs)
    s3 = synth.make_scenario(workload, seed=0, max_snapshots=3)
    t_dbs = float(s3.met["times"][1])
    g = F.Context(s3, F.PREC_FP32)
    g.run(beg_time=t_dbs - 30.0, end_time=t_dbs + 30.0)
    g.close()
    # batched form
    b = F.Batch(8)
    ctxs = [F.Context(synth.ensemble_member(100 + i, run_h=1.0, max_snapshots=2), F.PREC_FP32) for i in range(4)]
    for g in ctxs:
        b.add(g)
    for _ in range(3):
        b.step()
    b.sync()
    b.close()
    for g in ctxs:
        g.close()
    # gravity current and aggregation
    small = synth.make_scenario("small", seed=3, nx=64, ny=56, nz=20, run_h=0.5)
    g = F.Context(small, F.PREC_FP64)
    g.set_gravity_current(synth.gravity_current(small))
    g.run()
    g.close()
    agg = synth.make_scenario("small", seed=9, nx=64, ny=56, nz=20, nc=7, phimin=3.0, phimax=8.0,
                              aggregate=[0.2, 1000.0, 0.2], M0=1e7, run_h=0.25)
    synth.add_gas_class(agg)
    g = F.Context(agg, F.PREC_FP32)
    g.set_aggregation(synth.aggregation_inputs(agg))
    g.run()
    g.close()
    return F.kernel_launches() - n0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="cfg1")
    args = ap.parse_args()
    print(f"{run(args.workload)} kernel launches")


if __name__ == "__main__":
    main()
