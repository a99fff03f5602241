"""Drivers of the batched and serving forms on synthetic workloads.

ensemble   a batch of ensemble members (nx, ny ~ U[64,320], nz ~ U[20,60],
           4-20 classes, ...) advanced together through f3d_batch_* for a
           bounded number of batch steps: cell-class-steps/s of the batch.
serving    forecast requests (each an ensemble member with a duration
           U[dmin, dmax] h) arriving as a Poisson stream, submitted to the
           continuous-batching server (f3d_server_*) at their arrival times
           under an HBM admission cap; p50/p99 latency (arrival to result)
           and throughput, beside the latencies the same requests would see
           run one after another in the plain FP64 form (service times from
           the FP64 form's step and meteo-update rates measured here on a
           sample of the requests).

    python -m fall3d_gb300.serve ensemble [--members 64] [--steps 40]
    python -m fall3d_gb300.serve serving [--rate 2] [--window 600] [--cap-gb 150]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

import fall3d_gb300 as F
from fall3d_gb300 import synth


def ensemble(members=64, steps=40, run_h=12.0, seed=0, tune=True, warm=3):
    """Batch of ``members`` ensemble members: ``warm`` batch steps (meteo
    updates, autotune), then ``steps`` timed batch steps."""
    scen = [synth.ensemble_member(seed + i, run_h=run_h, max_snapshots=2) for i in range(members)]
    ctxs = [F.Context(s, F.PREC_FP32) for s in scen]
    b = F.Batch(members)
    for g in ctxs:
        b.add(g)
    for _ in range(warm):
        b.step()
    tuned = None
    if tune:
        tuned = b.autotune(reps=2)
        b.step()
    b.sync()
    bs0, cc0, _ = b.stats()
    t0 = time.perf_counter()
    for _ in range(steps):
        b.step()
    b.sync()
    t = time.perf_counter() - t0
    bs1, cc1, n = b.stats()
    cells = [s.grid["nx"] * s.grid["ny"] * s.grid["nz"] * s.grid["nc"] for s in scen]
    out = dict(members=members, batch_steps=bs1 - bs0, seconds=t, value=(cc1 - cc0) / t,
               cell_classes=int(sum(cells)), running=n,
               tile_shape=(tuned[0] if tuned else b.get_option(F.OPT_TILE)),
               autotune_ms=(tuned[1] if tuned else None))
    b.close()
    for g in ctxs:
        g.close()
    return out


def _fp64_rates(scens, steps=3):
    """Plain FP64 form on a few requests: (cell-class-steps/s of the step,
    seconds per meteo update per cell-class)."""
    step_rates, met_costs = [], []
    for s in scens:
        g = F.Context(s, F.PREC_FP64)
        g.source(0)
        t0 = time.perf_counter()
        g.meteo(0)
        g.sync()
        t_met = time.perf_counter() - t0
        g.step(1)
        g.sync()
        t0 = time.perf_counter()
        g.step(steps)
        g.sync()
        t = time.perf_counter() - t0
        cc = s.grid["nx"] * s.grid["ny"] * s.grid["nz"] * s.grid["nc"]
        step_rates.append(cc * steps / t)
        met_costs.append(t_met / cc)
        g.close()
    return float(np.mean(step_rates)), float(np.mean(met_costs))


def serving(rate=2.0, window=600.0, cap_gb=150.0, dmin=3.0, dmax=48.0, met_dt_h=12.0, seed=0,
            max_running=128, steps_per_poll=2, fp64_sample=2):
    rng = np.random.default_rng(seed)
    arrivals = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > window:
            break
        arrivals.append(t)
    n = len(arrivals)
    durs = rng.uniform(dmin, dmax, size=n)
    scen = [synth.ensemble_member(100_000 + seed * 10_000 + i, run_h=float(durs[i]), met_dt_h=met_dt_h)
            for i in range(n)]
    srv = F.Server(int(cap_gb * 1e9), max_running=max_running)
    ids = []
    t0 = time.monotonic()
    nxt = 0
    peak_running, peak_used = 0, 0
    while True:
        now = time.monotonic() - t0
        while nxt < n and arrivals[nxt] <= now:
            ids.append(srv.submit(scen[nxt]))
            nxt += 1
        running, queued = srv.progress(steps_per_poll)
        st = srv.stats()
        peak_running = max(peak_running, running)
        peak_used = max(peak_used, st["used_bytes"])
        if nxt == n and running == 0 and queued == 0:
            break
        if running == 0 and queued == 0 and nxt < n:
            time.sleep(max(0.0, arrivals[nxt] - (time.monotonic() - t0)))
    polls = [srv.poll(i) for i in ids]
    failed = [p for p in polls if p["state"] != F.Server.DONE]
    lat = np.array([p["t_done"] - (t0 + a) for p, a in zip(polls, arrivals)])
    makespan = max(p["t_done"] for p in polls) - t0
    st = srv.stats()
    steps = np.array([p["steps"] for p in polls])
    cc = np.array([s.grid["nx"] * s.grid["ny"] * s.grid["nz"] * s.grid["nc"] for s in scen], dtype=float)
    srv.close()
    # the same requests one after another in the plain FP64 form
    r_step, met_cost = _fp64_rates(scen[:fp64_sample])
    n_met = np.array([len([x for x in s.met["times"] if x < s.end_time]) for s in scen])
    service = cc * steps / r_step + n_met * cc * met_cost
    fin, seq_lat = 0.0, []
    for a, sv in zip(arrivals, service):
        fin = max(fin, a) + sv
        seq_lat.append(fin - a)
    seq_lat = np.array(seq_lat)
    return dict(
        requests=n, failed=len(failed), rate_per_s=rate, window_s=window, cap_gb=cap_gb,
        duration_h=[dmin, dmax], met_interval_h=met_dt_h,
        p50_latency_s=float(np.percentile(lat, 50)), p99_latency_s=float(np.percentile(lat, 99)),
        mean_latency_s=float(lat.mean()), makespan_s=float(makespan),
        value=float(st["cell_class_steps"] / makespan), cell_class_steps=float(st["cell_class_steps"]),
        peak_running=peak_running, peak_hbm_gb=peak_used / 1e9,
        fp64_sequential=dict(p50_latency_s=float(np.percentile(seq_lat, 50)),
                             p99_latency_s=float(np.percentile(seq_lat, 99)),
                             makespan_s=float(max(fin, 0.0)), step_rate=r_step,
                             meteo_s_per_cell_class=met_cost, sampled_requests=fp64_sample,
                             note="service times from the FP64 form's rates measured on the sampled "
                                  "requests; same step counts as served"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["ensemble", "serving"])
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--rate", type=float, default=2.0)
    ap.add_argument("--window", type=float, default=600.0)
    ap.add_argument("--cap-gb", type=float, default=150.0)
    ap.add_argument("--dmin", type=float, default=3.0)
    ap.add_argument("--dmax", type=float, default=48.0)
    ap.add_argument("--met-dt-h", type=float, default=12.0)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()
    if args.mode == "ensemble":
        print(json.dumps(ensemble(args.members, args.steps, seed=args.seed)))
    else:
        print(json.dumps(serving(args.rate, args.window, args.cap_gb, args.dmin, args.dmax, args.met_dt_h,
                                 args.seed)))


if __name__ == "__main__":
    main()
