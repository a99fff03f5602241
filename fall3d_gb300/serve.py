"""Drivers of the batched and serving forms on synthetic workloads.

ensemble   a batch of ensemble members (nx, ny ~ U[64,320], nz ~ U[20,60],
           4-20 classes, ...) advanced together through f3d_batch_* for a
           bounded number of batch steps: cell-class-steps/s of the batch.
ensemble_run  the same members each run to its end in one batch (the whole
           job), then each alone through f3d_run, compared bit for bit.
serving    forecast requests (each an ensemble member with a duration
           U[dmin, dmax] h) arriving as a Poisson stream, submitted to the
           continuous-batching server (f3d_server_*) at their arrival times
           under an HBM admission cap; p50/p99 latency (arrival to result)
           and throughput, beside the latencies of the same requests run
           one after another in the plain FP64 form (each run to its end and
           timed; a FIFO of the measured service times on the same arrivals).

    python -m fall3d_gb300.serve ensemble [--members 64] [--steps 40]
    python -m fall3d_gb300.serve ensemble-run [--members 64] [--run-h 12] [--met-dt-h-run 3]
    python -m fall3d_gb300.serve serving [--rate 2] [--window 600] [--cap-gb 150]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

import fall3d_gb300 as F
from fall3d_gb300 import synth


def ensemble(members=64, steps=40, run_h=12.0, seed=0, tune=True, warm=3, scen=None):
    """Batch of ``members`` ensemble members (or of the scenarios ``scen``):
    ``warm`` batch steps (meteo updates, autotune), then ``steps`` timed
    batch steps."""
    if scen is None:
        scen = [synth.ensemble_member(seed + i, run_h=run_h, max_snapshots=2) for i in range(members)]
    members = len(scen)
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


def ensemble_alone(members=64, steps=40, run_h=12.0, seed=0, warm=3, scen=None):
    """The members of ``ensemble`` (or the scenarios ``scen``) each alone in
    its own context, one after another (``warm`` steps, then ``steps`` timed
    steps each): the single-context rate on the batch's work,
    cell-class-steps/s."""
    import torch

    if scen is None:
        scen = [synth.ensemble_member(seed + i, run_h=run_h, max_snapshots=2) for i in range(members)]
    members = len(scen)
    cc_total, t_total = 0, 0.0
    for s in scen:
        g = F.Context(s, F.PREC_FP32)
        g.source(0)
        g.meteo(0)
        for _ in range(warm):
            g.step()
        g.sync()
        ext = torch.cuda.ExternalStream(g.stream_handle())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(steps):
            g.step()
        e1.record(ext)
        e1.synchronize()
        t_total += e0.elapsed_time(e1) / 1e3
        cc_total += s.grid["nx"] * s.grid["ny"] * s.grid["nz"] * s.grid["nc"] * steps
        g.close()
    return dict(members=members, steps=steps, seconds=t_total, value=cc_total / t_total)


def ensemble_run(members=64, run_h=12.0, met_dt_h=3.0, seed=0, alone=True):
    """The whole batched job: ``members`` ensemble members each run to its
    end (every source interval and meteo update; met snapshots every
    ``met_dt_h`` hours over the whole run) in one batch, timed from the
    first batch step to the last, autotune included; then, with ``alone``,
    each member run to its end in its own context through f3d_run, timed,
    and compared with its batched result (step count, c, cdry and cwet bit
    for bit)."""
    scen = [synth.ensemble_member(seed + i, run_h=run_h, met_dt_h=met_dt_h) for i in range(members)]
    ctxs = [F.Context(s, F.PREC_FP32) for s in scen]
    b = F.Batch(members)
    slots = [b.add(g) for g in ctxs]
    b.sync()
    t0 = time.perf_counter()
    for _ in range(3):
        b.step()
    tuned = b.autotune(reps=2)
    b.run()
    b.sync()
    t = time.perf_counter() - t0
    bs, cc, _ = b.stats()
    done = 0
    for sl in slots:
        try:
            done += int(b.poll(sl)[0] == F.Batch.DONE)
        except F.F3DError:  # the member's own error (its source or meteo update failed)
            pass
    cells = [s.grid["nx"] * s.grid["ny"] * s.grid["nz"] * s.grid["nc"] for s in scen]
    out = dict(members=members, run_h=run_h, met_interval_h=met_dt_h, done=done, batch_steps=bs, seconds=t, value=cc / t,
               cell_class_steps=cc, cell_classes=int(sum(cells)), tile_shape=tuned[0])
    if alone:
        t_alone, same, steps = 0.0, 0, []
        for i, s in enumerate(scen):
            g = F.Context(s, F.PREC_FP32)
            g.sync()
            t1 = time.perf_counter()
            g.run()
            g.sync()
            t_alone += time.perf_counter() - t1
            sa, sb = g.state(), ctxs[i].state()
            fa, fb = g.fields(), ctxs[i].fields()
            steps.append(sa["iiter"])
            same += int(sa["iiter"] == sb["iiter"] and sa["time"] == sb["time"] and
                        all(np.array_equal(fa[k], fb[k], equal_nan=True) for k in ("c", "cdry", "cwet")))
            g.close()
        out["alone"] = dict(seconds=t_alone, value=cc / t_alone, members_bitwise_equal=same,
                            steps_min=int(min(steps)), steps_max=int(max(steps)))
        out["batched_over_alone"] = t_alone / t
    b.close()
    for g in ctxs:
        g.close()
    return out


def fp64_sequential(scens, arrivals):
    """The same requests one after another in the plain FP64 form: each is
    run to its end (context creation, f3d_run with its meteorology and
    sources, the deposit maps read back) and timed; a single FIFO server
    then gives request i the latency finish_i - arrival_i with finish_i =
    max(finish_{i-1}, arrival_i) + service_i."""
    service = []
    for s in scens:
        t0 = time.perf_counter()
        g = F.Context(s, F.PREC_FP64)
        g.run()
        g.outputs()
        g.close()
        service.append(time.perf_counter() - t0)
    lat, fin = fifo_latencies(arrivals, service)
    return np.array(service), lat, fin


def fifo_latencies(arrivals, service):
    """One server taking requests in arrival order: request i finishes at
    finish_i = max(finish_{i-1}, arrival_i) + service_i; returns the
    latencies finish_i - arrival_i and the last finish time."""
    fin, lat = 0.0, []
    for a, sv in zip(arrivals, service):
        fin = max(fin, a) + sv
        lat.append(fin - a)
    return np.array(lat), fin


def serving(rate=2.0, window=600.0, cap_gb=150.0, dmin=3.0, dmax=48.0, met_dt_h=12.0, seed=0,
            max_running=128, steps_per_poll=2, fp64=True):
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
    srv.close()
    out = dict(
        requests=n, failed=len(failed), rate_per_s=rate, window_s=window, cap_gb=cap_gb,
        duration_h=[dmin, dmax], met_interval_h=met_dt_h,
        p50_latency_s=float(np.percentile(lat, 50)), p99_latency_s=float(np.percentile(lat, 99)),
        mean_latency_s=float(lat.mean()), makespan_s=float(makespan),
        value=float(st["cell_class_steps"] / makespan), cell_class_steps=float(st["cell_class_steps"]),
        peak_running=peak_running, peak_hbm_gb=peak_used / 1e9)
    if fp64:
        # the same requests one after another in the plain FP64 form, run and timed
        service, seq_lat, seq_makespan = fp64_sequential(scen, arrivals)
        out["fp64_sequential"] = dict(
            p50_latency_s=float(np.percentile(seq_lat, 50)), p99_latency_s=float(np.percentile(seq_lat, 99)),
            makespan_s=float(seq_makespan), service_s_total=float(service.sum()), requests_run=len(service),
            note="every request run to its end in the FP64 form, one after another; latency from the "
                 "measured service times and the same arrivals")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["ensemble", "ensemble-run", "serving"])
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--rate", type=float, default=2.0)
    ap.add_argument("--window", type=float, default=600.0)
    ap.add_argument("--cap-gb", type=float, default=150.0)
    ap.add_argument("--dmin", type=float, default=3.0)
    ap.add_argument("--dmax", type=float, default=48.0)
    ap.add_argument("--met-dt-h", type=float, default=12.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--run-h", type=float, default=12.0)
    ap.add_argument("--met-dt-h-run", type=float, default=3.0, help="met interval of ensemble-run")
    args = ap.parse_args()
    if args.mode == "ensemble":
        print(json.dumps(ensemble(args.members, args.steps, seed=args.seed)))
    elif args.mode == "ensemble-run":
        print(json.dumps(ensemble_run(args.members, args.run_h, args.met_dt_h_run, seed=args.seed)))
    else:
        print(json.dumps(serving(args.rate, args.window, args.cap_gb, args.dmin, args.dmax, args.met_dt_h,
                                 args.seed)))


if __name__ == "__main__":
    main()
