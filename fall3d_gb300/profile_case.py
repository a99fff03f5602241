"""Runs a few steps of a named workload through the context API: the case
that profiler captures of the step kernels run.

    python -m fall3d_gb300.profile_case [--workload cfg1] [--steps 3]
                                        [--precision 32] [--fused 1] [--tile 0]
                                        [--time]

With --time, the steps after the first are timed per kernel with CUDA
events and printed as milliseconds per launch, then two meteo updates are
timed on the host clock.
"""
from __future__ import annotations

import argparse
import time

import fall3d_gb300 as F
from fall3d_gb300 import synth


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="cfg1")
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--precision", type=int, default=32)
    ap.add_argument("--fused", type=int, default=1)
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--classes", type=int, default=0, help="override the class count")
    ap.add_argument("--time", action="store_true", help="print per-kernel times")
    args = ap.parse_args()
    over = {"max_snapshots": 2}
    if args.classes:
        over["nc"] = args.classes
    s = synth.make_scenario(args.workload, seed=0, **over)
    g = F.Context(s, args.precision)
    if args.precision == 32:
        g.set_option(F.OPT_FUSED, args.fused)
        g.set_option(F.OPT_TILE, args.tile)
    g.source(0)
    g.meteo(0)
    if args.time:
        g.step(1)
        g.profile(True)
        g.step(args.steps - 1)
        g.sync()
        for name, (n, ms) in sorted(g.profile_read().items(), key=lambda kv: -kv[1][1]):
            print(f"  {name:12s} {n:4d} launches {ms / max(n, 1):9.4f} ms/launch")
        for snap in (1, 0):  # a meteo update: upload, coefficient chain, settling velocities
            t0 = time.perf_counter()
            g.meteo(snap)
            g.sync()
            print(f"  meteo update {time.perf_counter() - t0:9.4f} s (host clock, upload included)")
    else:
        g.step(args.steps)
    g.sync()
    st = g.state()
    print(f"{args.workload}: {st['iiter']} steps, dt {st['dt']:.3f} s, outmass {st['outmass']:.6e}")


if __name__ == "__main__":
    main()
