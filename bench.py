"""Throughput of the FALL3D transport step on GB300 (cell-class-steps/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: the 400x300x50 grid with 16 particle classes (phi -2..6), seeded
synthetic meteorology with a k^-5/3 wind perturbation and a precipitation
band (wet deposition on), Suzuki column 15 km, MER 1e7 kg/s.  A step is one
pass of Sources/Fall3d.f90:112-117 over all classes (setsrc, sizloop with
setbcc, advection, diffusion, wet and dry deposition, clip, cmass2d).

``value``    precision form (binary32 stencil, binary64 budgets/accum/finddt)
             with inputs resident in HBM, timed with CUDA events on the
             context's stream over K steps; the state (0.4 GB of c alone) is
             larger than the 126 MB L2, so no flush is needed between steps.
``e2e``      the same metric through the C ABI's time loop (f3d_run) from
             host buffers over eight DBS intervals (4 h simulated):
             meteorology and sources uploaded by the loop when their
             intervals begin, each meteo update after the first computed
             while the previous interval steps (F3D_OPT_PREFETCH; the same
             window with every update made when due is reported beside it),
             the deposit maps (LOAD, COL_MASS, C_GRND) read back at the end,
             all inside the timed region.
``forms``    the plain binary64 form on the same workload; the batched form
             (64 ensemble members, nx, ny ~ U[64,320], nz ~ U[20,60], 4-20
             classes, one persistent launch per batch step, 30 timed batch
             steps, beside the same members run alone one after another);
             the served form on a bounded sample of the Poisson request
             stream (p50/p99 latency, beside the same requests run to their
             end one after another in the FP64 form).
``accuracy_vs_fp64``  relative L2 / Linf error of every output of the
             precision form against the FP64 form over the e2e window, and
             the mass drift |massvol+massdep+outmass-erumass|/erumass.
``--impl reference`` times the reference's own Fortran path (translated to C
by oracle/ref_translate.py, oracle/_ref) on the host cores, one process per
class group as in its MPI class decomposition, with a serial (1 core)
sample beside it; the CPU oracle port stands in where no translation exists.
Multi-GPU: classes and scenarios are independent, so N GPUs run N replicas
of the workload with no collective ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "cfg1"
METRIC = "cell-class-steps/s"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


E2E_INTERVALS = 8  # DBS intervals of the end-to-end window (4 h of the 24-h forecast)


def _scenario(max_snapshots=E2E_INTERVALS + 1):
    from fall3d_gb300 import synth

    return synth.make_scenario(WORKLOAD, seed=0, max_snapshots=max_snapshots)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "", 1).isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


# Algorithmic bytes per cell-class of each kernel (element size S).  The
# whole step (and so the fused step kernel) has the fixed contract figure
# 2S (read and write c) + S (vset) + 7S/nc (the class-shared fields vx, vy,
# vz, rho, rkhor, rkh1, rkver, amortised over the classes) = 3S + 7S/nc,
# whatever the kernel actually moves.  The per-routine kernels read every
# operand once and write every output once, met fields per class.
def kernel_bytes_per_cell_class(S, nc):
    return {"step_fused": 3 * S + 7 * S / nc, "advctzc": 4 * S, "advctx": 3 * S, "advcty": 3 * S,
            "diffz": 4 * S, "diffx": 4 * S, "diffy": 4 * S, "clip": 2 * S}


def cpu_baseline(threads, steps=2):
    """The CPU oracle on this host's cores on a bounded sample: one meteo
    update (timed separately), ``steps`` full steps of the workload on all
    cores (OpenMP over classes), then one step on one core (the serial
    build's rate)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib

    s = _scenario(max_snapshots=2)
    o = oracle_lib.OracleCtx(s, nthreads=threads)
    o.source(0)
    t0 = time.perf_counter()
    o.meteo(0)
    t_met = time.perf_counter() - t0
    o.step()  # warm-up
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    t = time.perf_counter() - t0
    o.set_threads(1)
    t0 = time.perf_counter()
    o.step()
    t1 = time.perf_counter() - t0
    units = s.cell_classes * steps
    o.close()
    return {"value": units / t, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{WORKLOAD} 400x300x50x16: {steps} full steps after one meteo update "
                      f"(meteo update {t_met:.1f} s, not in the rate); oracle -O2 -ffp-contract=off, "
                      f"OpenMP over classes",
            "serial_1core": {"value": s.cell_classes / t1, "unit": METRIC, "cores": 1,
                             "sample": "one full step on one core after the sample above"}}


def _reference_lib():
    """The translated reference (oracle/_ref), built if needed; None with the
    reason when it cannot be."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    try:
        import ref_translate

        ref_translate.build()
        return True, None
    except Exception as e:  # no sources and no translation: the port stands in
        return False, str(e).splitlines()[0] if str(e) else type(e).__name__


def run_reference(args, rank, world):
    """The reference's CPU path on the host cores.  With the translated
    reference available (the reference's own Fortran, oracle/_ref): one
    process per class group as in the reference's MPI class decomposition,
    after the serial set-up and a serial sample; otherwise the CPU oracle
    port with OpenMP over classes."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    s = _scenario(max_snapshots=2)
    nc = s.grid["nc"]
    ok, why = _reference_lib()
    extra = {}
    if ok:
        import ref_driver

        ngrp = max(1, min(threads, nc))
        r = ref_driver.time_class_parallel(s, ngrp, args.steps, serial_steps=2, budget_s=45.0)
        par, ser = r["parallel"], r["serial"]
        done, t = par["steps"], par["seconds"]
        v = par["cell_class_steps"] / t
        kind, cores = "reference", ngrp
        form = (f"the reference's own Fortran (translated to C, gcc -O2 -ffp-contract=off), "
                f"{ngrp} processes over class groups (Sources/Parallel.F90 localdim/globalindex)")
        sample = (f"{done} steps of {WORKLOAD} per class group, all groups started together, after one "
                  f"untimed step; set-up: the serial meteo update ({r['meteo_s']:.1f} s, not in the rate)")
        extra["serial_1core"] = {"value": ser["cell_class_steps"] / ser["seconds"], "unit": METRIC, "cores": 1,
                                 "steps": ser["steps"], "seconds": ser["seconds"],
                                 "sample": "full steps over every class in one process (the serial build)"}
        extra["meteo_update_s"] = r["meteo_s"]
    else:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_lib

        o = oracle_lib.OracleCtx(s, nthreads=threads)
        o.source(0)
        o.meteo(0)
        for _ in range(args.warmup):
            o.step()
        done = 0
        t0 = time.perf_counter()
        while done < args.steps:
            o.step()
            done += 1
            if time.perf_counter() - t0 > 150.0:
                break
        t = time.perf_counter() - t0
        o.close()
        v = s.cell_classes * done / t
        kind, cores = "port", threads
        form = "CPU oracle (binary64), OpenMP over classes, all host cores"
        sample = f"{done} full steps of {WORKLOAD} after one meteo update"
        extra["reference_unavailable"] = why
    line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": world, "steps": done,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / done, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "grid": [400, 300, 50], "classes": nc, "form": form},
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line.update(extra)
    print(json.dumps(line), flush=True)


def captured_traffic(kernel, workload=WORKLOAD, root=ROOT):
    """DRAM bytes (read + write) of one launch of ``kernel`` from the
    committed ncu capture (profiles/ncu_traffic.json), valid only while the
    step kernel's source is the one that was captured (its SHA-256 is stored
    beside the figure); returns (bytes or None, where the figure comes from)."""
    tpath = os.path.join(root, "profiles", "ncu_traffic.json")
    if not os.path.exists(tpath):
        return None, "no capture"
    try:
        rec = json.load(open(tpath)).get(workload, {})
        kpath = os.path.join(root, "fall3d_gb300", "csrc", "f3d_fused2.cu")
        sha = hashlib.sha256(open(kpath, "rb").read()).hexdigest()
    except (OSError, ValueError):
        return None, "no capture"
    if rec.get("kernel_sha256") != sha:
        return None, "stale: the kernel source changed since the capture"
    return rec.get(kernel), "ncu capture of this kernel source"


def max_over_ranks_of(x, dist=None, device="cpu"):
    """The largest of every rank's x (the job's time is its slowest rank's)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_step, steps, world, ms):
    """Whole-job throughput: every rank runs its own replica of the workload
    (weak scaling), the job takes the slowest rank's time ms."""
    return units_per_step * steps * world / (ms / 1e3)


def run_ours(args, rank, world, local_rank):
    import torch
    import fall3d_gb300 as F

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        return max_over_ranks_of(x, dist, "cuda")

    s = _scenario()
    units_per_step = s.cell_classes

    # ---------------- precision form, inputs resident in HBM ----------------
    g = F.Context(s, F.PREC_FP32)
    g.source(0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g.meteo(0)
    meteo_s = time.perf_counter() - t0
    for _ in range(max(args.warmup, 3)):
        g.step()
    g.sync()
    ext = torch.cuda.ExternalStream(g.stream_handle())
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local_rank)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    n0 = F.kernel_launches()
    ev0.record(ext)
    for _ in range(args.steps):
        g.step()
    ev1.record(ext)
    ev1.synchronize()
    n_launch = F.kernel_launches() - n0
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    ms = max_over_ranks(ms)
    value = job_rate(units_per_step, args.steps, world, ms)

    # per-kernel durations with CUDA events on the same stream
    g.profile(True)
    for _ in range(args.steps):
        g.step()
    prof = g.profile_read()
    g.profile(False)
    g.close()

    # ---------------- plain binary64 form ----------------
    g64 = F.Context(s, F.PREC_FP64)
    g64.source(0)
    g64.meteo(0)
    k64 = max(2, min(args.steps, 6))
    for _ in range(2):
        g64.step()
    g64.sync()
    ext64 = torch.cuda.ExternalStream(g64.stream_handle())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext64)
    for _ in range(k64):
        g64.step()
    e1.record(ext64)
    e1.synchronize()
    ms64 = e0.elapsed_time(e1)
    value64 = units_per_step * k64 / (ms64 / 1e3)
    g64.close()

    # ---------------- end to end through the C ABI time loop ----------------
    # One forecast window of E2E_INTERVALS meteorological intervals (30
    # simulated minutes each): the loop uploads each DBS snapshot (from
    # page-locked host buffers) and the sources when their intervals begin,
    # computes each meteo update after the first one while the previous
    # interval steps (F3D_OPT_PREFETCH), steps, logs the budget every 10
    # simulated minutes, and the deposit maps are read back at the end.
    from fall3d_gb300 import _abi

    def pinned(a):  # a numpy view of page-locked host memory holding a copy of a
        a = np.ascontiguousarray(a)
        t = torch.empty(a.shape, dtype=torch.float64 if a.dtype == np.float64 else torch.int32, pin_memory=True)
        v = t.numpy()
        v[...] = a
        pinned.keep.append(t)
        return v

    pinned.keep = []
    met_h = {k: (pinned(np.asarray(v, dtype=np.float64)) if k not in ("times", "time_lag") else v)
             for k, v in s.met.items()}
    met = _abi.make_met(met_h)
    src = _abi.make_src(s.src)
    window = float(s.met["times"][E2E_INTERVALS] - s.met["times"][0])
    ge = F.Context(s, F.PREC_FP32)
    ge.run(max_steps=2, met=met, src=src)  # warm-up (allocations, first meteo)
    ge.close()
    ge = F.Context(s, F.PREC_FP32)
    ge.set_option(F.OPT_PREFETCH, 1)  # the look-ahead's second met set, allocated with the context
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    log = ge.run(end_time=window, met=met, src=src)
    outs = ge.outputs()
    t_e2e = time.perf_counter() - t0
    t_e2e = max_over_ranks(t_e2e)
    st = ge.state()
    e2e_steps = st["iiter"]
    # the same window with every meteo update made when it is due
    gn = F.Context(s, F.PREC_FP32)
    gn.set_option(F.OPT_PREFETCH, 0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gn.run(end_time=window, met=met, src=src)
    gn.outputs()
    t_e2e_due = max_over_ranks(time.perf_counter() - t0)
    gn.close()
    f32_fields = ge.fields() if (rank == 0 and not args.no_forms) else None
    ge.close()
    nx, ny, nz, nc = s.grid["nx"], s.grid["ny"], s.grid["nz"], s.grid["nc"]
    times = s.met["times"]
    # snapshots the loop read: those whose time a step started at or after
    # (the run stops once time >= window, before the next snapshot's update)
    n_meteo = int(np.sum(times < window)) if len(times) else 1
    n_meteo = max(1, min(n_meteo, len(times)))
    met_bytes = (6 * nx * ny * nz + 6 * nx * ny) * 8
    src_bytes = int(s.src["nsou"][0]) * (3 * 4 + nc * 8)
    h2d = (n_meteo * met_bytes + src_bytes) / e2e_steps
    d2h = (3 * nx * ny * 8 + len(log["iiter"]) * 5 * 8) / e2e_steps
    e2e_value = units_per_step * e2e_steps * world / t_e2e

    # ---------------- roofline of the dominant kernel ----------------
    peak, peak_kind = _peaks()
    dom = max(prof.items(), key=lambda kv: kv[1][1]) if prof else ("none", (1, 0.0))
    dom_name, (dom_n, dom_ms) = dom
    bpc = kernel_bytes_per_cell_class(4, nc).get(dom_name)
    roof = None
    if bpc and dom_n:
        cells = units_per_step if dom_name != "clip" else (nx + 2) * (ny + 2) * (nz + 2) * nc
        alg_bytes = bpc * cells
        avg_ms = dom_ms / dom_n
        achieved = alg_bytes / (avg_ms / 1e3) / 1e9
        traffic, traffic_note = captured_traffic(dom_name)
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_note, "kernel": dom_name,
                "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": avg_ms,
                "peak_source": f"{peak_kind} hbm_gbs"}
    step_bytes = 12 + 28 / nc  # binary32 algorithmic bytes per cell-class-step
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": [nx, ny, nz], "classes": nc,
                   "form": "precision (binary32 stencil, binary64 budgets/accum/finddt)",
                   "l2": "state larger than L2 (no flush needed)", "parallelism": f"replicas{world}"},
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": e2e_steps, "meteo_updates": n_meteo,
                "value_updates_when_due": units_per_step * e2e_steps * world / t_e2e_due,
                "window": f"{E2E_INTERVALS} DBS intervals ({window:.0f} s simulated) through f3d_run from "
                          f"page-locked host buffers, each meteo update after the first computed while the "
                          f"previous interval steps"},
        "gpu_launches": int(n_launch),
        "clocks": clk,
        "roofline": roof,
        "step_roofline": {"alg_bytes_per_cell_class_step": step_bytes,
                          "achieved_gbs": value / world * step_bytes / 1e9,
                          "frac": value / world * step_bytes / 1e9 / peak},
        "forms": {"fp64_plain": {"value": value64, "ms_per_step": ms64 / k64, "steps": k64},
                  "fp32_over_fp64": value / world / value64},
        "kernels_ms_per_step": {k: v[1] / max(1, v[0]) for k, v in prof.items()},
        "meteo_update_s": meteo_s,
    }
    if rank == 0 and not args.no_forms:
        # precision form vs the plain FP64 form over the same window: every
        # output, and the mass drift |massvol+massdep+outmass-erumass|/erumass
        g64 = F.Context(s, F.PREC_FP64)
        log64 = g64.run(end_time=window, met=met, src=src)
        outs64, f64_fields, st64 = g64.outputs(), g64.fields(), g64.state()
        g64.close()
        err = {}
        pairs = [("LOAD", outs["load"], outs64["load"]), ("COL_MASS", outs["col_mass"], outs64["col_mass"]),
                 ("C_GRND", outs["c_grnd"], outs64["c_grnd"]), ("c", f32_fields["c"], f64_fields["c"]),
                 ("cdry", f32_fields["cdry"], f64_fields["cdry"]), ("cwet", f32_fields["cwet"], f64_fields["cwet"])]
        for name, a32, a64 in pairs:
            d = np.asarray(a32, dtype=np.float64) - a64
            n64 = float(np.linalg.norm(a64.ravel()))
            m64 = float(np.max(np.abs(a64)))
            err[name] = {"rel_l2": float(np.linalg.norm(d.ravel())) / n64 if n64 > 0 else 0.0,
                         "rel_linf": float(np.max(np.abs(d))) / m64 if m64 > 0 else 0.0}

        def drift(lg):
            eru = lg["erumass"][-1]
            return abs(lg["massvol"][-1] + lg["massdep"][-1] + lg["outmass"][-1] - eru) / eru if eru else 0.0

        line["accuracy_vs_fp64"] = {
            "window": f"{window:.0f} s simulated ({e2e_steps} steps, identical step sequence: "
                      f"{st['iiter'] == st64['iiter'] and st['dt'] == st64['dt']})",
            "errors": err, "mass_drift_fp32": drift(log), "mass_drift_fp64": drift(log64),
            "massvol_rel_diff": abs(log["massvol"][-1] - log64["massvol"][-1]) / abs(log64["massvol"][-1])}
        from fall3d_gb300 import serve

        try:
            fb = serve.ensemble(members=64, steps=30)
            fb["over_fp64_plain"] = fb["value"] / value64
            alone = serve.ensemble_alone(members=64, steps=10)
            fb["members_alone"] = alone
            fb["over_members_alone"] = fb["value"] / alone["value"]
            line["forms"]["fp32_batched"] = fb
            # the batch machinery on grids of the single-context size: four
            # scenarios of the benchmarked workload (seeds 1-4) batched and alone
            from fall3d_gb300 import synth as _synth

            big = [_synth.make_scenario(WORKLOAD, seed=i + 1, max_snapshots=2) for i in range(4)]
            fu = serve.ensemble(steps=10, scen=big)
            fa = serve.ensemble_alone(steps=10, scen=big)
            line["forms"]["fp32_batched_4x" + WORKLOAD] = {
                "value": fu["value"], "members_alone": fa["value"], "over_members_alone": fu["value"] / fa["value"],
                "over_single_context": fu["value"] / (value / world), "tile_shape": fu["tile_shape"]}
        except Exception as e:
            line["forms"]["fp32_batched"] = {"error": str(e)}
        try:
            sv = serve.serving(rate=2.0, window=10.0, dmin=0.3, dmax=4.8, met_dt_h=1.0)
            sv["sample"] = ("Poisson 2 req/s for 10 s, ensemble-member requests with durations "
                            "U(0.3, 4.8) h (one tenth of the serving config's 3-48 h), hourly met; "
                            "the FP64 baseline runs every request to its end, one after another")
            line["forms"]["served"] = sv
        except Exception as e:
            line["forms"]["served"] = {"error": str(e)}
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            line["cpu_baseline"] = cpu_baseline(os.cpu_count() or 1)
        except Exception as e:  # reported, never silently replaced
            line["cpu_baseline"] = {"error": str(e)}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the accuracy check and the batched and served forms")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
