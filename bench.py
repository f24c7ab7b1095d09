"""Benchmark of the GB300 GeoClaw patch update (cell-updates/s, FP64).

Workload (the plain GPU drop-in microbenchmark): one uniform level of
4096 patches of 32 x 32 cells (64 x 64 patches, 2048 x 2048 = 4,194,304
cells, dx = 1 m) over a seeded diamond-square DEM (Hurst 0.8, 30 m relief)
with a 5 m deep, 40 m wide carved channel; dam-break start (surface 10 m
above the bed for x < 600 m, dry beyond); Manning n = 0.035; dry tolerance
1e-3 m; FP64. A step is one level step: the fused patch update of every
patch (b4step2, step2, CFL, src2) followed by the same-level ghost copy.

value  - cell-updates/s with the level resident in HBM (inputs 170 MB, larger
         than the 129 MB L2, so no flush between steps).
e2e    - the same through the C ABI with host buffers: gf_level_step_host
         copies q in (pinned, Fortran layout), steps, copies q out.
roofline - HBM roofline of the patch kernel (56 algorithmic bytes per
         interior cell-update) against the measured copy bandwidth, plus the
         FP64 issue roofline it is actually bound by.
cpu_baseline - the CPU oracle (Fortran-faithful C restatement, OpenMP over
         patches) on a bounded sample of the same level.

--impl reference times the reference CPU path (the oracle port; the
reference's Fortran cannot be built on this image) on all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-updates/s"
BYTES_PER_CELL_UPDATE = 56  # read h, hu, hv, b; write h, hu, hv (FP64)
# Per tile shape of the mx = 32 update (threads, slices per band), from one ncu
# capture each of the launch this bench times first in its kernel-only loop
# (update launch 24 of `--steps 20 --warmup 3`, the same state): DRAM
# traffic (dram__bytes_read.sum + dram__bytes_write.sum, against 234.9 MB
# algorithmic) and FP64 warp instructions (sm__inst_executed_pipe_fp64.sum;
# x 32 lanes / 4 194 304 cell-updates = FP64 issue slots per cell-update)
NCU_COUNTS = {(256, 7): (170.886912e6 + 62.938880e6, 29.892596e6),
              (384, 9): (170.445312e6 + 66.367744e6, 29.903210e6)}
NCU_DEFAULT_TILE = (384, 9)
M = 32
NPX = NPY = 64
DX = 1.0
DT = 0.03  # CFL ~ 0.4-0.6 on this state
SEED = 2024
MTHBC = (1, 1, 1, 1)  # zero-order extrapolation, as the reference dam_break example


def workload():
    from geoflood_gb300 import synth

    q, aux, py, px = synth.uniform_dam_break_level(NPX, NPY, M, DX, seed=SEED, x_dam=600.0)
    return q, aux, py, px


def config():
    """The workload both arms run (the same dict in both JSON lines)."""
    return {"workload": "dam-break level step, 4096 patches of 32x32, fractal DEM + channel",
            "patches": NPX * NPY, "mx": M, "cells": NPX * NPY * M * M, "dt_s": DT,
            "l2": "inputs 170 MB > L2, no flush"}


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", os.environ.get("GF_BENCH_GPU_INDEX", "0"), "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_state_at_timing(q, aux, nsteps):
    """The level state at the start of the GPU arm's timed steps: nsteps
    level steps (update at DT, then the same-level ghost fill with the
    bench's boundary rule) of the CPU oracle on the whole level, from the
    same initial state, so the CPU samples time the state the GPU times."""
    import oracle
    from geoflood_gb300 import Phys, synth

    phys = Phys()
    qa = np.ascontiguousarray(q).copy()
    aus = np.ascontiguousarray(aux)
    nbr, xl, yl = synth.brick_layout(NPY, NPX, M, DX)
    oracle.level_ghost_fill(qa, aus, nbr, xl, yl, DX, DX, 0.0, mthbc=MTHBC, phys=phys)
    for k in range(nsteps):
        oracle.level_update(qa, aus, DX, DX, k * DT, DT, phys, nthreads=0)
        oracle.level_ghost_fill(qa, aus, nbr, xl, yl, DX, DX, (k + 1) * DT, mthbc=MTHBC, phys=phys)
    return qa


def cpu_oracle_rate(q, aux, seconds=12.0, rows=8, threads=0):
    """Time the CPU oracle on whole patch rows of the level state the GPU
    arm times (cpu_state_at_timing); repeats one step until `seconds` have
    elapsed."""
    import oracle

    n = rows * NPX
    start_row = NPY // 2 - rows // 2
    sl = slice(start_row * NPX, start_row * NPX + n)
    qs = np.ascontiguousarray(q[sl])
    aus = np.ascontiguousarray(aux[sl])
    from geoflood_gb300 import Phys

    phys = Phys()
    oracle.load()
    cells = 0
    t0 = time.perf_counter()
    reps = 0
    while True:
        work = qs.copy()
        oracle.level_update(work, aus, DX, DX, 0.0, DT, phys, nthreads=threads)
        cells += n * M * M
        reps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    return cells / el, cores, f"{rows} patch rows ({n} patches) per step, {reps} steps"


def buffered_hook_rate(ctx, q, aux, dx, dt, steps=3, buffer_len=1024):
    """The plain per-patch GPU drop-in as ForestClaw drives the reference's
    GPU build: every patch of the level handed to the buffered
    single_step_update hook (gf_step_buffer_update, as cudaclaw_update,
    src/fc2d_cpu_cuda/fc2d_cpucuda.cpp:410-495) one at a time from its own
    host array, flushed every buffer_len patches (1024, the reference
    examples' buffer_length). Returns cell-updates/s over `steps` level
    steps after one untimed step."""
    import geoflood_gb300 as gf

    n, m = q.shape[0], q.shape[1] - 4
    qs = [np.array(q[k]) for k in range(n)]
    auxs = [np.ascontiguousarray(aux[k]) for k in range(n)]
    buf = gf.StepBuffer(ctx, buffer_len)

    def level_step():
        mc = 0.0
        for k in range(n):
            mc = max(mc, buf.update(k, n, qs[k], auxs[k], dx, dx, 0.0, dt))
        return mc

    level_step()
    t0 = time.perf_counter()
    for _ in range(steps):
        level_step()
    el = time.perf_counter() - t0
    buf.close()
    return steps * n * m * m / el


def lone_patch_latency_us(ctx, q, aux, reps=50):
    """One wet 32 x 32 patch through gf_patch_update (host buffers, one call):
    the median latency of a lone patch, the drop-in's single-patch path."""
    k = int(np.argmax((q[:, 2:-2, 2:-2, 0] > 1e-3).sum(axis=(1, 2))))
    qk, ak = np.array(q[k]), np.ascontiguousarray(aux[k])
    for _ in range(5):
        ctx.patch_update(qk.copy(), ak, DX, DX, 0.0, DT)
    ts = []
    for _ in range(reps):
        w = qk.copy()
        t0 = time.perf_counter()
        ctx.patch_update(w, ak, DX, DX, 0.0, DT)
        ts.append(time.perf_counter() - t0)
    return 1e6 * float(np.median(ts))


def reduce_over_ranks(dist, values: dict, ops: dict) -> dict:
    """Combine per-rank results on every rank: ops[k] is "max", "min" or
    "sum". Replicas share no data; this only aggregates their timings and
    counts (device tensors under NCCL, CPU tensors under gloo)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return dict(values)
    import torch

    red = {"max": dist.ReduceOp.MAX, "min": dist.ReduceOp.MIN, "sum": dist.ReduceOp.SUM}
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    out = {}
    for k, v in values.items():
        t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=red[ops[k]])
        out[k] = float(t.item())
    return out


def shard(n: int, rank: int, world: int) -> list:
    """Items of rank `rank` when n independent items (scenarios, forests)
    are dealt round-robin to `world` replicas."""
    return list(range(rank, n, world))


SERVED_SEED = 4242


def _pinned(shape):
    import torch

    return torch.empty(int(np.prod(shape)), dtype=torch.float64,
                       pin_memory=True).numpy().reshape(shape)


def served_stream(args):
    """Served scenario stream: Poisson arrivals of flood scenarios
    (finest-level cells log-uniform in [1e4, 4e6], mx drawn from {8,16,32},
    fractal valley DEM with a channel, hydrograph peak 10-500 m^3/s rising
    over 0.5-2 h, n ~ U[0.02, 0.08], horizon 1-6 h; times multiplied by
    --served-time-scale, 1 = the horizons as drawn) through the
    continuous-batching server at 80 % of the capacity measured in a
    saturated calibration window."""
    import threading

    import geoflood_gb300 as gf
    from geoflood_gb300 import synth

    n = args.served_scenarios
    ts = args.served_time_scale
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    g = np.random.default_rng(SERVED_SEED)
    cells = np.exp(g.uniform(np.log(1e4), np.log(4e6), n))
    seeds = [SERVED_SEED + 1 + k for k in range(n)]
    params = [synth.flood_scenario_params(seeds[k], float(cells[k]), time_scale=ts)
              for k in range(n)]

    def make(k):
        sc = synth.flood_scenario(seeds[k], float(cells[k]), time_scale=ts, alloc=_pinned)
        return sc, _pinned(sc.q.shape)

    def wet_fraction(q, drytol):
        return float((q[:, 2:-2, 2:-2, 0] > drytol).mean())

    # warm the shared DEM lattices so generation keeps ahead of arrivals
    synth.flood_scenario(1, 3e6, mx=32, time_scale=ts)
    synth.flood_scenario(2, 3e6, mx=32, time_scale=ts)

    lanes = tuple(int(float(v)) for v in args.served_lanes.split(",") if v.strip())
    srv = gf.Server(device=dev, reserve_sms=args.served_reserve_sms, lanes=lanes,
                    cull_dry=not args.served_no_cull, split_sizes=not args.served_no_split)
    srv.start()

    # -- calibration: a saturated batch; throughput over a bounded window
    #    (until half of it has finished, or --served-cal-seconds), the rest
    #    cancelled
    ncal = min(16, n)
    cal_items = [make(k) for k in range(ncal)]
    st_a = srv.stats()
    t0 = srv.clock()
    cal_ids = [srv.submit(sc, qo) for sc, qo in cal_items]
    while True:
        st = srv.stats()
        t_now = srv.clock()
        left = st["active"] + st["queued"]
        if left <= ncal // 2 or t_now - t0 >= args.served_cal_seconds:
            break
        time.sleep(0.002)
    cap = (st["cell_updates"] - st_a["cell_updates"]) / (t_now - t0)
    cal_info = [srv.poll(i) for i in cal_ids]
    for i in cal_ids:
        if srv.poll(i)["state"] not in ("done", "failed", "cancelled"):
            srv.cancel(i)
    for i in cal_ids:
        srv.wait(i, timeout=600)
        srv.release(i)
    del cal_items
    steps_per_sim_s = (sum(i["steps"] for i in cal_info) /
                       max(sum(i["t"] for i in cal_info), 1e-9))
    est_work = float(np.mean([cells[k] * params[k]["horizon"] * steps_per_sim_s for k in range(n)]))
    rate = 0.8 * cap / est_work if args.served_rate is None else float(args.served_rate)
    load = rate * est_work / cap
    gaps = np.random.default_rng(SERVED_SEED + 7).exponential(1.0 / rate, n)
    arrivals = np.cumsum(gaps) - gaps[0]
    # size-stratified sample for the isolated re-runs
    ns = min(args.served_sample, n)
    order = np.argsort(cells)
    sample = sorted({int(order[int(round(f * (n - 1)))]) for f in np.linspace(0.0, 1.0, ns)})

    def run_stream(arrivals, count):
        """The first `count` scenarios at the given arrival times: producer
        threads keep generated scenarios ahead of the arrivals (numpy
        releases the GIL in the array work)."""
        ready, cond, nxt, taken = {}, threading.Condition(), [0], [0]
        ahead = 48

        def producer():
            while True:
                with cond:
                    while nxt[0] < count and nxt[0] >= taken[0] + ahead:
                        cond.wait()
                    if nxt[0] >= count:
                        return
                    k = nxt[0]
                    nxt[0] += 1
                item = make(k)
                with cond:
                    ready[k] = item
                    cond.notify_all()

        def take(k):
            with cond:
                while k not in ready:
                    cond.wait()
                taken[0] = k + 1
                cond.notify_all()
                return ready.pop(k)

        workers = [threading.Thread(target=producer, daemon=True)
                   for _ in range(max(2, min(8, (os.cpu_count() or 4) // 2)))]
        for w in workers:
            w.start()
        with cond:
            while len(ready) < min(ahead, count) and any(w.is_alive() for w in workers):
                cond.wait(0.05)
        st0 = srv.stats()
        t_start = srv.clock()
        ids, pending, infos, outs, late, mx_of = {}, [], {}, {}, 0, {}
        qout_of, drytol_of, wet0, wet1 = {}, {}, {}, {}

        def sweep(block=False):
            for k in list(pending):
                info = srv.wait(ids[k], timeout=3600) if block else srv.poll(ids[k])
                if info["state"] in ("done", "failed", "cancelled"):
                    infos[k] = info
                    pending.remove(k)
                    wet1[k] = wet_fraction(qout_of.pop(k), drytol_of[k])
                    if k not in sample:
                        srv.release(ids[k])

        for k in range(count):
            sc, qo = take(k)
            t_arr = t_start + arrivals[k]
            while srv.clock() < t_arr:
                time.sleep(min(0.002, max(t_arr - srv.clock(), 0.0)))
            if srv.clock() - t_arr > 0.01:
                late += 1
            ids[k] = srv.submit(sc, qo)
            mx_of[k] = sc.mx
            drytol_of[k] = sc.phys.dry_tolerance
            wet0[k] = wet_fraction(sc.q, sc.phys.dry_tolerance)
            qout_of[k] = qo
            pending.append(k)
            if k in sample:
                outs[k] = qo
            del sc, qo
            sweep()
        for w in workers:
            w.join()
        sweep(block=True)
        for k in sample:
            if k in ids:
                srv.release(ids[k])
        return (infos, outs, late, mx_of, st0, srv.stats(), t_start,
                max(i["t_done"] for i in infos.values()), wet0, wet1)

    infos, outs, late, mx_of, st0, st1, t_start, t_end, wet0, wet1 = run_stream(arrivals, n)
    low = None
    if args.served_low_load:
        # the first half of the stream again at 50 % load (arrival gaps x 1.6)
        low = run_stream(arrivals[: n // 2] * 1.6, n // 2)
    failed = sum(1 for i in infos.values() if i["state"] != "done")
    lat = np.array([i["t_done"] - i["t_submit"] for i in infos.values()])
    work = sum(i["cell_updates"] for i in infos.values())
    served_rate = work / (t_end - t_start)
    # wet cell-updates: each scenario's cell-updates times the mean of its
    # start and end wet fractions
    wet_work = sum(i["cell_updates"] * 0.5 * (wet0[k] + wet1[k]) for k, i in infos.items())

    # -- isolated re-runs of a size-stratified sample: latency alone, same bits
    slow, slow_low, same, detail = [], [], True, []
    for k in sample:
        sc, qo = make(k)
        sid = srv.submit(sc, qo)
        ik = srv.wait(sid, timeout=3600)
        t_iso = ik["t_done"] - ik["t_submit"]
        t_mix = infos[k]["t_done"] - infos[k]["t_submit"]
        slow.append(t_mix / t_iso)
        same &= bool(np.array_equal(qo, outs[k])) and ik["steps"] == infos[k]["steps"]
        if low is not None and k in low[0]:
            slow_low.append((low[0][k]["t_done"] - low[0][k]["t_submit"]) / t_iso)
            same &= bool(np.array_equal(qo, low[1][k]))
        detail.append({"cells": int(sc.cells), "mx": sc.mx, "lane": ik["lane"], "steps": ik["steps"],
                       "isolated_s": t_iso, "mixed_s": t_mix, "wet_end": wet1[k],
                       "queued_s": infos[k]["t_admit"] - infos[k]["t_submit"]})
        srv.release(sid)
    srv.stop()
    srv.close()

    # -- the plain per-patch drop-in (the buffered hook) on the same work mix
    ctx = gf.Context(dev)
    rate_mx = {}
    for mx in (8, 16, 32):
        sc = synth.flood_scenario(SERVED_SEED, 2.0e6, mx=mx, time_scale=ts)
        ctx.set_phys(0, sc.phys)
        rate_mx[mx] = buffered_hook_rate(ctx, sc.q, sc.aux, sc.dx, 0.2, steps=2)
    ctx.close()
    plain_time = sum(i["cell_updates"] / rate_mx[mx_of[k]] for k, i in infos.items())
    plain_rate = work / plain_time
    out = {
        "value": served_rate, "unit": METRIC, "scenarios": n, "failed": failed,
        "p50_latency_s": float(np.percentile(lat, 50)),
        "p99_latency_s": float(np.percentile(lat, 99)),
        "slowdown_vs_isolated": {"p50": float(np.percentile(slow, 50)),
                                 "p99": float(np.percentile(slow, 99)), "max": float(max(slow)),
                                 "sample": len(sample), "detail": detail},
        "alone_equals_mix": same,
        "wet_fraction": wet_work / max(work, 1),
        "wet_cell_updates_per_s": wet_work / (t_end - t_start),
        "plain_per_patch": {"value": plain_rate, "unit": METRIC,
                            "per_mx": {str(k): v for k, v in rate_mx.items()},
                            "note": "buffered single_step_update hook (gf_step_buffer_update, "
                                    "buffer 1024) with host buffers, weighted by the stream's "
                                    "work per mx"},
        "vs_plain_per_patch": served_rate / plain_rate,
        "capacity": {"value": cap, "unit": METRIC, "scenarios": ncal, "window_s": t_now - t0,
                     "note": "saturated batch, until half of it had finished or the window "
                             "closed"},
        "arrival_rate_per_s": rate, "offered_load": load, "late_submissions": late,
        "stream_seconds": t_end - t_start, "cell_updates": work,
        "launches": st1["launches"] - st0["launches"], "rounds": st1["rounds"] - st0["rounds"],
        "peak_device_bytes": st1["bytes_peak"],
        "workload": f"{n} flood scenarios, cells log-uniform [1e4, 4e6], mx in {{8,16,32}}, "
                    f"dx 5 m, horizons 1-6 h x{ts:.4g}",
    }
    if low is not None:
        lat_low = np.array([i["t_done"] - i["t_submit"] for i in low[0].values()])
        out["at_50pct_load"] = {
            "scenarios": n // 2, "arrival_rate_per_s": rate / 1.6,
            "p50_latency_s": float(np.percentile(lat_low, 50)),
            "p99_latency_s": float(np.percentile(lat_low, 99)),
            "slowdown_vs_isolated": {"p50": float(np.percentile(slow_low, 50)),
                                     "p99": float(np.percentile(slow_low, 99)),
                                     "max": float(max(slow_low)), "sample": len(slow_low)},
            "note": "the first half of the stream, arrival gaps x 1.6"}
    return out


def run_reference(args):
    """Reference arm: the reference's CPU patch update (oracle port) on all host threads."""
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    q, aux, _, _ = workload()
    import oracle

    from geoflood_gb300 import Phys

    oracle.load()
    # the state the GPU arm's timed steps start from
    q = cpu_state_at_timing(q, aux, max(args.warmup, 3))
    rows = 4
    n = rows * NPX
    sl = slice((NPY // 2) * NPX, (NPY // 2) * NPX + n)
    qs = np.ascontiguousarray(q[sl])
    aus = np.ascontiguousarray(aux[sl])
    phys = Phys()
    for _ in range(args.warmup):
        w = qs.copy()
        oracle.level_update(w, aus, DX, DX, 0.0, DT, phys, nthreads=0)
    times = []
    for _ in range(args.steps):
        w = qs.copy()
        t0 = time.perf_counter()
        oracle.level_update(w, aus, DX, DX, 0.0, DT, phys, nthreads=0)
        times.append(time.perf_counter() - t0)
    cells = n * M * M
    v = cells * len(times) / sum(times)
    cores = os.cpu_count() or 1
    line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": config(),
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": cores, "kind": "port",
                             "sample": f"{rows} patch rows ({n} patches) of the timed state per "
                                       "step; the oracle port (no Fortran compiler here)"},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def _sig(x, n=4):
    """x rounded to n significant digits (floats only)."""
    if isinstance(x, float) and x != 0.0 and np.isfinite(x):
        return float(f"{x:.{n}g}")
    return x


def compact(r: dict) -> dict:
    """The one-line record: the contract's keys and a short summary of every
    leg (the full figures go to --detail)."""
    keep = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
            "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "gpu_launches",
            "config", "e2e", "cpu_baseline")
    out = {k: r[k] for k in keep if k in r}
    out["value"], out["ms_per_step"] = _sig(r["value"]), _sig(r["ms_per_step"])
    if "e2e" in out:
        out["e2e"] = dict(out["e2e"], value=_sig(out["e2e"]["value"]))
    if "cpu_baseline" in out:
        out["cpu_baseline"] = dict(out["cpu_baseline"], value=_sig(out["cpu_baseline"]["value"]))
    rl = r["roofline"]
    out["roofline"] = {"bound": rl["bound"], "achieved": _sig(rl["achieved"]), "peak": rl["peak"],
                       "unit": rl["unit"], "frac": _sig(rl["frac"], 3), "traffic": int(rl["traffic"])}
    ck = r.get("clocks") or {}
    out["clocks"] = {"sm_mhz": ck.get("sm_mhz"), "sm_max_mhz": ck.get("sm_max_mhz"),
                     "reasons": ck.get("reasons")}
    fp = r.get("fp64")
    if fp:
        out["fp64"] = {"frac_of_measured_dfma": _sig(fp["frac_of_measured_dfma"], 3),
                       "peak_gops": _sig(fp["peak_dfma_gops"])}
    pp = r.get("plain_per_patch")
    if pp:
        out["plain_per_patch"] = {"value": _sig(pp["value"]), "lone_patch_us": _sig(pp["lone_patch_us"])}
    sv = r.get("served")
    if sv:
        out["served"] = {"value": _sig(sv["value"]), "scenarios": sv["scenarios"],
                         "horizons": sv["workload"].split("horizons ")[-1],
                         "p50_s": _sig(sv["p50_latency_s"], 3), "p99_s": _sig(sv["p99_latency_s"], 3),
                         "slowdown_p50": _sig(sv["slowdown_vs_isolated"]["p50"], 3),
                         "slowdown_p99": _sig(sv["slowdown_vs_isolated"]["p99"], 3),
                         "wet_frac": _sig(sv["wet_fraction"], 3),
                         "vs_plain_per_patch": _sig(sv["vs_plain_per_patch"], 3),
                         "alone_equals_mix": sv["alone_equals_mix"]}
    bt = r.get("batched")
    if bt:
        out["batched"] = {"value": _sig(bt["value"]),
                          "vs_one_by_one": _sig(bt.get("speedup_vs_one_by_one"), 3),
                          "equal": bt.get("batch_equals_one_by_one")}
    fs = r.get("forest")
    if fs:
        out["forest"] = {"value": _sig(fs["value"]),
                         "regrid_mismatches": fs.get("regrid_parity", {}).get("mismatching_regrids"),
                         "subcycled_batch_x": _sig(fs["to_60s"]["subcycled_batch"]["speedup_vs_one_by_one"], 3)}
    sa = r.get("served_amr")
    if sa:
        sl = sa.get("slowdown_vs_isolated", {})
        out["served_amr"] = {"value": _sig(sa["value"]), "p99_s": _sig(sa.get("p99_latency_s"), 3),
                             "slowdown_p99": _sig(sl.get("p99"), 3)}
    if r.get("large"):
        out["large"] = _sig(r["large"]["value"])
    if r.get("dem"):
        out["dem"] = _sig(r["dem"]["value"])
    return out


def run_gpu(args):
    import torch

    import geoflood_gb300 as gf
    from geoflood_gb300 import synth

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    q, aux, py, px = workload()
    ncell = NPX * NPY * M * M
    ctx = gf.Context(local, gf.Phys())
    # tile shapes per patch size, measured on this device (process-wide choice)
    tiles = ctx.autotune(reps=3) if not (args.no_autotune or args.tiles) else None
    for spec in filter(None, args.tiles.split(",")):
        mx_s, thr, lat = (int(v) for v in spec.split(":"))
        gf.Context.set_tile(mx_s, 0, thr)
        gf.Context.set_tile(mx_s, 1, lat)
    lev = gf.Level(ctx, q.shape[0], M, 1)
    lev.set_geometry(DX, DX)
    lev.upload(q, aux)
    nbr, xl, yl = synth.brick_layout(py, px, M, DX)
    lev.set_layout(nbr, xl, yl)
    lev.set_bc(MTHBC)
    lev.ghost_fill(0.0)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    launches_per_step = 2  # patch update + ghost fill
    clock = [0.0]

    def step():
        lev.step_async(clock[0], DT)
        clock[0] += DT
        lev.ghost_fill_async(clock[0])

    for _ in range(max(args.warmup, 3)):
        step()
    lev.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
    maxcfl = lev.sync()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # kernel-only timing of the patch update (no ghost fill) for the roofline
    with torch.cuda.stream(stream):
        k0 = torch.cuda.Event(enable_timing=True)
        k1 = torch.cuda.Event(enable_timing=True)
        k0.record(stream)
        nk = max(3, min(args.steps, 10))
        for _ in range(nk):
            lev.step_async(0.0, DT)
        k1.record(stream)
    lev.sync()
    kernel_ms = k0.elapsed_time(k1) / nk
    clk = clocks.stop()
    ms = reduce_over_ranks(dist, {"ms": ms}, {"ms": "max"})["ms"]

    # e2e through the C ABI with host buffers (pinned, Fortran layout); the
    # host array carries the filled ghost cells, as ForestClaw's storage does
    qh = torch.empty(q.size, dtype=torch.float64, pin_memory=True).numpy().reshape(q.shape)
    lev.upload(q, aux)
    lev.ghost_fill(0.0)
    qh[...] = lev.download()
    for _ in range(2):
        lev.step_host(qh, 0.0, DT)
    ne = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        h0 = torch.cuda.Event(enable_timing=True)
        h1 = torch.cuda.Event(enable_timing=True)
        h0.record(stream)
        for _ in range(ne):
            lev.step_host(qh, 0.0, DT)
        h1.record(stream)
    torch.cuda.synchronize()
    e2e_wall = (time.perf_counter() - t0) / ne
    e2e_ms = max(h0.elapsed_time(h1) / ne, 1e3 * e2e_wall)
    e2e_ms = reduce_over_ranks(dist, {"ms": e2e_ms}, {"ms": "max"})["ms"]
    qbytes = q.size * 8

    plain_v = buffered_hook_rate(ctx, q, aux, DX, DT)
    lone_us = lone_patch_latency_us(ctx, q, aux)

    hbm_peak, peak_kind = load_peaks()
    tile32 = (384, 9)
    tsel = next((t for t in (tiles or []) if t["mx"] == M), None)
    if tsel is not None:
        tile32 = tuple(tsel["tiles"][tsel["best_throughput"]][:2])
    elif args.tiles:
        for spec in filter(None, args.tiles.split(",")):
            mx_s, thr, _ = (int(v) for v in spec.split(":"))
            if mx_s == M:
                tile32 = {0: (256, 7), 1: (256, 5), 2: (384, 7), 3: (384, 9)}.get(thr, tile32)
    traffic, fp64_warp_inst = NCU_COUNTS.get(tile32, NCU_COUNTS[NCU_DEFAULT_TILE])
    algo = BYTES_PER_CELL_UPDATE * ncell
    achieved = algo / (kernel_ms * 1e-3) / 1e9
    rates = fp64_rates()
    fp64 = None
    if rates:
        fp64 = {"bound": "fp64 issue", "peak_dfma_gops": rates["dfma"] / 1e9,
                "ddiv_gops": rates["ddiv"] / 1e9, "dsqrt_gops": rates["dsqrt"] / 1e9,
                "ffma_gops": rates["ffma"] / 1e9,
                "kernel_cell_updates_per_s": ncell / (kernel_ms * 1e-3),
                "peak_source": "measured live (gf_measure_fp64_rates)"}
        # FP64 issue slots (warp instructions x 32 lanes) per cell-update of
        # this workload, from the ncu capture of the same kernel: the achieved
        # FP64 issue rate follows from the live kernel time
        ops = fp64_warp_inst * 32 / float(ncell)
        ach = ops * ncell / (kernel_ms * 1e-3) / 1e9
        fp64.update({"lane_ops_per_cell_update": ops, "achieved_gops": ach,
                     "frac_of_measured_dfma": ach / (rates["dfma"] / 1e9),
                     "ops_source": "ncu sm__inst_executed_pipe_fp64.sum of this kernel on "
                                   "this workload x 32 lanes / cell-updates (one capture)"})
    result = {
        "metric": METRIC, "value": world * ncell / (ms * 1e-3), "unit": METRIC,
        "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": config(),
        "max_cfl_last_step": maxcfl,
        "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
        "e2e": {"value": world * ncell / (e2e_ms * 1e-3), "unit": METRIC,
                "h2d_bytes_per_step": qbytes, "d2h_bytes_per_step": qbytes + 16},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic, "tile": list(tile32),
                     "traffic_unit": "bytes per launch",
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum "
                                       "of one launch (one capture)",
                     "algorithmic_bytes_per_launch": algo,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "kernel_ms": kernel_ms,
                     "note": "FP64-issue bound, not HBM bound: see fp64"},
        "fp64": fp64,
        "clocks": clk,
        "tiles": tiles,
        "plain_per_patch": {"value": plain_v, "unit": METRIC, "lone_patch_us": lone_us,
                            "note": "buffered single_step_update hook over the whole level "
                                    "(gf_step_buffer_update, buffer 1024, one host array per "
                                    "patch); lone_patch_us: one gf_patch_update call"},
    }
    if rank == 0 and not args.no_served:
        result["served"] = served_stream(args)
    if rank == 0 and not args.no_forest:
        result["forest"] = forest_leg(args, local)
        result["batched"] = batched_leg(args, local)
        result["served_amr"] = fserved_leg(args, local)
    if rank == 0 and not args.no_large:
        result["large"] = large_leg(args, local)
    if rank == 0 and not args.no_dem:
        result["dem"] = dem_leg(args, local)
    if rank == 0:
        if not args.no_cpu_baseline:
            qt = cpu_state_at_timing(q, aux, max(args.warmup, 3))
            v, cores, sample = cpu_oracle_rate(qt, aux, seconds=args.cpu_seconds)
            result["cpu_baseline"] = {"value": v, "unit": METRIC, "cores": cores, "kind": "port",
                                      "sample": sample}
        if args.detail:
            Path(args.detail).write_text(json.dumps(result, indent=1))
        print(json.dumps(compact(result), separators=(",", ":")))
    lev.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


def forest_dambreak_config(mx=16, lmin=1, lmax=3, seed=SEED):
    """The CPU dam break as a forest: 2000 x 1000 m as a 2 x 1 brick of
    1000 m blocks, levels 1..3 (dx 31.25 m .. 7.8125 m at mx = 16), bump-and-
    ramp bed, surface 10 m above the bed for x < 600 m, dry beyond, n =
    0.035, walls; refinement follows moving water (flowgrade on momentum
    > 1 m^2/s up to level 3), regrid every 2 steps."""
    import geoflood_gb300 as gf
    from geoflood_gb300 import synth

    nbx, nby = 2, 1
    dx0 = 1000.0 / mx
    nx, ny = nbx * mx << lmax, nby * mx << lmax
    dxf = dx0 / (1 << lmax)
    b = synth.bump_ramp_dem(nx, ny, dxf, dxf, seed=seed)
    x = (np.arange(nx) + 0.5) * dxf
    q = np.zeros((ny, nx, 3))
    q[..., 0] = np.where(x[None, :] < 600.0, 10.0, 0.0)
    rf = gf.Refine(wave_tolerance=1e9, flowgrades=((1.0, 2, 1, lmax),))
    phys = gf.Phys(manning_coefficient=(0.035,), manning_break=(1e10,))
    return dict(mx=mx, nbx=nbx, nby=nby, lmin=lmin, lmax=lmax, dx0=dx0, b=b, q=q, rf=rf,
                phys=phys, mthbc=(3, 3, 3, 3), regrid=2)


def regrid_parity(ctx, c, attempts, resync, exact=False):
    """Config-1 dam break driven step by step on the GPU forest and the
    oracle's forest driver with the outstyle-1 control of
    fc2d_geoclaw_run.c:229-395 (advance-one-step, reject / retake, a regrid
    every `regrid` accepted steps). resync = True: before every regrid the
    oracle restarts from the GPU's leaves and state, so each regrid is
    compared from identical states (tags and the regridded patch list);
    resync = False: both sides run free, each with its own dt control. Returns
    (regrids, regrids whose patch lists differ)."""
    import geoflood_gb300 as gf
    from oracle import forest as of

    if exact:
        ctx.set_fp_contract(False)
    G = gf.Forest(ctx, c["mx"], c["nbx"], c["nby"], c["lmin"], c["lmax"], c["dx0"], c["dx0"],
                  c["b"], c["q"], mthbc=c["mthbc"], regrid_interval=0, refine=c["rf"])
    G.init()
    O = of.Forest(c["mx"], c["nbx"], c["nby"], c["lmin"], c["lmax"], c["dx0"], c["dx0"], c["b"],
                  c["q"], phys=c["phys"], mthbc=c["mthbc"], regrid_interval=0, rf=c["rf"])
    O.init()
    level_factor = float(1 << (c["lmax"] - c["lmin"]))
    desired, max_cfl = 0.9, 1.0
    state = {"G": [0.0, 5.0, 0], "O": [0.0, 5.0, 0]}   # t, dt_minlevel, accepted

    def attempt(name):
        t, dtm, acc = state[name]
        dt = dtm / level_factor
        if name == "G":
            cfl = G.step(t, dt)
            G.accept(cfl <= max_cfl)
        else:
            snap = O.snapshot()
            cfl = O.step(t, dt)
            if cfl > max_cfl:
                O.restore(snap)
        if cfl > max_cfl:
            state[name] = [t, dtm * desired / cfl, acc]
            return False
        state[name] = [t + dt, dtm * desired / cfl if cfl > 0.0 else dtm, acc + 1]
        return state[name][2] % c["regrid"] == 0

    regrids = mism = 0
    for _ in range(attempts):
        due = attempt("G")
        if resync:
            if due:
                O.adopt(G.patches(), G.download())
                t = state["G"][0]
                G.regrid(t)
                O.regrid(t)
                regrids += 1
                mism += int(not np.array_equal(G.patches(), O.patches()))
        else:
            due_o = attempt("O")
            if due or due_o:
                if due:
                    G.regrid(state["G"][0])
                if due_o:
                    O.regrid(state["O"][0])
                regrids += 1
                mism += int(not (due and due_o and np.array_equal(G.patches(), O.patches())))
    G.close()
    if exact:
        ctx.set_fp_contract(True)
    return regrids, mism


def forest_leg(args, dev=0):
    """Config-1 dam break (AMR forest) on the GPU forest and on the oracle's
    forest driver (CPU, same rules), same number of accepted steps."""
    import geoflood_gb300 as gf
    import oracle
    from oracle import forest as of

    c = forest_dambreak_config()
    steps = args.forest_steps
    ctx = gf.Context(dev)
    ctx.set_phys(0, c["phys"])
    F = gf.Forest(ctx, c["mx"], c["nbx"], c["nby"], c["lmin"], c["lmax"], c["dx0"], c["dx0"],
                  c["b"], c["q"], mthbc=c["mthbc"], regrid_interval=c["regrid"], refine=c["rf"])
    F.init()
    t0 = time.perf_counter()
    st = F.run(1e9, 1, 5.0, 0.9, 1.0, max_steps=steps)
    gpu_s = time.perf_counter() - t0
    gpu_patches = F.patches()
    # one frame of the final leaves in the reference's ASCII format
    with tempfile.TemporaryDirectory() as td:
        t0 = time.perf_counter()
        F.write_frame(1, td)
        frame_s = time.perf_counter() - t0
        frame_bytes = sum(os.path.getsize(os.path.join(td, n)) for n in os.listdir(td))
    frame_cells = int(len(gpu_patches)) * c["mx"] * c["mx"]
    F.close()
    # the same dam break to a 60 s horizon with and without subcycling
    horizon = {}
    for sub in (False, True):
        G = gf.Forest(ctx, c["mx"], c["nbx"], c["nby"], c["lmin"], c["lmax"], c["dx0"], c["dx0"],
                      c["b"], c["q"], mthbc=c["mthbc"], regrid_interval=c["regrid"], refine=c["rf"],
                      subcycle=sub)
        G.init()
        t0 = time.perf_counter()
        hs = G.run(60.0, 1, 5.0, 0.9, 1.0)
        sec = time.perf_counter() - t0
        G.close()
        horizon["subcycled" if sub else "advance_one_step"] = {
            "seconds": sec, "coarse_or_global_steps": hs["steps"], "rejects": hs["rejects"],
            "cell_updates": hs["cell_updates"], "value": hs["cell_updates"] / sec, "unit": METRIC}
    # 16 subcycled dam-break forests (bed seeds differ) to the 60 s horizon:
    # side by side in one batched call vs one after another
    from geoflood_gb300.forest import batch_run
    nsub = 16
    cs = [forest_dambreak_config(seed=SEED + 40 + k) for k in range(nsub)]

    def sub_forests():
        fs = []
        for cc in cs:
            G = gf.Forest(ctx, cc["mx"], cc["nbx"], cc["nby"], cc["lmin"], cc["lmax"], cc["dx0"], cc["dx0"],
                          cc["b"], cc["q"], mthbc=cc["mthbc"], regrid_interval=cc["regrid"], refine=cc["rf"],
                          subcycle=True)
            G.init()
            fs.append(G)
        return fs

    fs = sub_forests()
    t0 = time.perf_counter()
    for G in fs:
        G.run(60.0, 1, 5.0, 0.9, 1.0)
    seq_s = time.perf_counter() - t0
    seq = [(G.patches(), G.download(), G.stats()["cell_updates"]) for G in fs]
    for G in fs:
        G.close()
    fs = sub_forests()
    t0 = time.perf_counter()
    batch_run(fs, 60.0, 1, 5.0, 0.9, 1.0)
    bat_s = time.perf_counter() - t0
    work = sum(G.stats()["cell_updates"] for G in fs)
    same = all(np.array_equal(P, G.patches()) and np.array_equal(q[:, 2:-2, 2:-2], G.download()[:, 2:-2, 2:-2])
               for (P, q, _), G in zip(seq, fs))
    for G in fs:
        G.close()
    horizon["subcycled_batch"] = {
        "forests": nsub, "value": work / bat_s, "unit": METRIC, "seconds": bat_s,
        "one_by_one": {"value": work / seq_s, "seconds": seq_s},
        "speedup_vs_one_by_one": seq_s / bat_s, "batch_equals_one_by_one": bool(same),
        "note": "gf_forest_batch_run of subcycled forests: forests spanning the same levels step "
                "in shared launches, each group's coarse step a CUDA graph"}
    rp = regrid_parity(ctx, c, steps, resync=True)
    fr = regrid_parity(ctx, c, steps, resync=False, exact=True)
    ctx.close()
    oracle.load()
    O = of.Forest(c["mx"], c["nbx"], c["nby"], c["lmin"], c["lmax"], c["dx0"], c["dx0"], c["b"],
                  c["q"], phys=c["phys"], mthbc=c["mthbc"], regrid_interval=c["regrid"],
                  rf=c["rf"])
    O.init()
    t0 = time.perf_counter()
    O.run(1e9, 1, 5.0, 0.9, 1.0, max_steps=steps)
    cpu_s = time.perf_counter() - t0
    return {
        "workload": "dam break forest, 2x1 blocks of 1000 m, mx 16, levels 1-3, "
                    f"{steps} step attempts (accepted + rejected), regrid every 2",
        "value": st["cell_updates"] / gpu_s, "unit": METRIC, "seconds": gpu_s,
        "steps": st["steps"], "rejects": st["rejects"], "regrids": st["regrids"],
        "patches_end": int(len(gpu_patches)), "patches_max": st["npatch_max"],
        "cpu_oracle": {"value": O.cell_updates / cpu_s, "unit": METRIC, "seconds": cpu_s,
                       "cores": 1, "kind": "port",
                       "note": "oracle forest driver (Python tree + C kernels, one thread)"},
        "regrid_parity": {"regrids": rp[0], "mismatching_regrids": rp[1],
                          "exact_free_run": {"regrids": fr[0], "mismatching_regrids": fr[1]},
                          "note": "production build, oracle restarted from the GPU state before "
                                  "each regrid; exact_free_run: contraction-free build and oracle "
                                  "each on their own"},
        "to_60s": horizon,
        "ascii_frame": {"cells": frame_cells, "bytes": frame_bytes, "seconds": frame_s,
                        "cells_per_s": frame_cells / frame_s, "MB_per_s": frame_bytes / frame_s / 1e6,
                        "note": "gf_forest_write_ascii: leaf download + fort.t/fort.q text"},
    }


def dem_leg(args, dev=0):
    """DEM ingestion: a 2049 x 2049-node fractal DEM at 2 m over 4096 m x
    4096 m and a 1025 x 1025-node inset at 0.5 m, both read from type-3
    files, cell-averaged (setaux) at every level 0-5 of a 4 x 4 brick of
    32 x 32 patches (cells 32 m .. 1 m, 22.4 M cells plus halos), against the
    oracle's C restatement of the same integrals on one host thread."""
    import geoflood_gb300 as gf
    from geoflood_gb300 import synth
    from geoflood_gb300.topo import Topo
    from oracle import topo as ot

    A = np.round(synth.diamond_square(11, 0.8, SEED + 11) * 6.0 + 20.0, 3)
    B = np.round(synth.diamond_square(10, 0.8, SEED + 12) * 2.0 + 20.0, 3)
    grids = [(A, 0.0, 0.0, 2.0), (B, 1024.0, 1024.0, 0.5)]
    mx, nb, lmax, dx0 = 32, 4, 5, 32.0
    out = {"workload": "DEM 2049^2 nodes at 2 m + 1025^2 inset at 0.5 m (type-3 files), "
                       "setaux at levels 0-5 of 4x4 blocks of mx 32 (cells 32 m..1 m)"}
    with tempfile.TemporaryDirectory() as td:
        paths = []
        for k, (z, x0, y0, d) in enumerate(grids):
            p = os.path.join(td, "dem%d.tt3" % k)
            with open(p, "w") as f:
                f.write("%d ncols\n%d nrows\n%r xlower\n%r ylower\n%r cellsize\n-9999 nodata\n"
                        % (z.shape[1], z.shape[0], x0, y0, d))
                np.savetxt(f, z[::-1], fmt="%.3f")
            paths.append(p)
        fbytes = sum(os.path.getsize(p) for p in paths)
        t0 = time.perf_counter()
        topo = Topo()
        for p in paths:
            topo.read_file(p, 3)
        read_s = time.perf_counter() - t0
    # the oracle integrates the same nodes (the readers are pinned by the tests)
    ts = ot.TopoSet([topo.grid(k) for k in range(len(topo))])
    ctx = gf.Context(dev)
    ctx.set_phys(0, gf.Phys(sea_level=20.0))
    cells = sum((nb * mx << l) ** 2 for l in range(lmax + 1))
    F = gf.Forest(ctx, mx, nb, nb, 0, lmax, dx0, dx0, None, None)
    t0 = time.perf_counter()
    F.set_topo(topo)                      # first call: DEM upload + all levels
    first_s = time.perf_counter() - t0
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        F.set_topo(topo)
    dev_s = (time.perf_counter() - t0) / reps
    F.close()
    # parity on one level, and the oracle over every level
    n2, d2, ext = nb * mx << 2, dx0 / 4, nb * mx * dx0
    gpu_l2 = topo.raster(ctx, n2, n2, 2, 0.0, 0.0, d2, d2, ext, ext)
    ctx.close()
    equal = False
    t0 = time.perf_counter()
    for l in range(lmax + 1):
        n = nb * mx << l
        r = ts.raster(n, n, 2, 0.0, 0.0, dx0 / (1 << l), dx0 / (1 << l), ext, ext)
        if l == 2:
            equal = bool(np.array_equal(r, gpu_l2))
    cpu_s = time.perf_counter() - t0
    out.update({
        "value": cells / dev_s, "unit": "cell-averages/s", "cells": cells, "seconds": dev_s,
        "first_call_seconds": first_s,
        "read": {"bytes": fbytes, "seconds": read_s, "MB_per_s": fbytes / read_s / 1e6},
        "level2_equal_to_oracle": equal,
        "cpu_oracle": {"value": cells / cpu_s, "unit": "cell-averages/s", "seconds": cpu_s,
                       "cores": 1, "kind": "port", "sample": "all six levels"},
    })
    return out


def batched_leg(args, dev=0):
    """Batched AMR (config 3): forests with mx drawn from {8, 16, 32},
    levels 2..5, target patch counts log-uniform in [50, 5000], fractal
    valley DEM, reservoir + inflow hydrograph, n ~ U[0.02, 0.08], regrid every
    4 steps; a bounded simulated time. The same forests run once as one
    batch (shared launches, device-side control, captured rounds) and once
    one after another with Forest.run; a sample is checked bit for bit."""
    import geoflood_gb300 as gf
    from geoflood_gb300 import synth
    from geoflood_gb300.forest import batch_run

    n = args.batch_forests
    T = args.batch_time
    g = np.random.default_rng(SEED + 3)
    targets = np.exp(g.uniform(np.log(50), np.log(5000), n))
    specs = [synth.flood_forest(SEED + 100 + k, float(targets[k])) for k in range(n)]
    ctx = gf.Context(dev)

    def build():
        fs = []
        for k, sp in enumerate(specs):
            ctx.set_phys(1 + k, sp["phys"])
            F = gf.Forest(ctx, sp["mx"], sp["nbx"], sp["nby"], sp["minlevel"], sp["maxlevel"],
                          sp["dx0"], sp["dy0"], sp["aux"], sp["q"], mthbc=sp["mthbc"],
                          regrid_interval=sp["regrid_interval"], refine=sp["refine"],
                          phys_slot=1 + k)
            F.set_hydrograph(*sp["hydro"])
            F.init()
            fs.append(F)
        return fs

    A = build()
    patches0 = [F.npatch for F in A]
    t0 = time.perf_counter()
    bst = batch_run(A, T, 1, 1.6, 0.9, 1.0)
    el_b = time.perf_counter() - t0
    sample = list(range(0, n, max(1, n // 8)))
    ref = {k: (A[k].patches(), A[k].download(), A[k].stats()) for k in sample}
    work = sum(F.stats()["cell_updates"] for F in A)
    pmax = [F.stats()["npatch_max"] for F in A]
    for F in A:
        F.close()
    B = build()
    t0 = time.perf_counter()
    for F in B:
        F.run(T, 1, 1.6, 0.9, 1.0)
    el_s = time.perf_counter() - t0
    work_s = sum(F.stats()["cell_updates"] for F in B)
    same = all(np.array_equal(ref[k][0], B[k].patches())
               and np.array_equal(ref[k][1][:, 2:-2, 2:-2], B[k].download()[:, 2:-2, 2:-2])
               and ref[k][2]["steps"] == B[k].stats()["steps"] for k in sample)
    for F in B:
        F.close()
    ctx.close()
    # the oracle's forest driver (Python tree, C kernels on all host cores)
    # on a bounded sample: two forests of the batch, 4 step attempts each
    import oracle
    from oracle import forest as of
    cu_o, s_o, picks = 0, 0.0, [int(np.argsort(patches0)[n // 4]), int(np.argsort(patches0)[n // 2])]
    for k in picks:
        sp = specs[k]
        O = of.Forest(sp["mx"], sp["nbx"], sp["nby"], sp["minlevel"], sp["maxlevel"], sp["dx0"], sp["dy0"],
                      sp["aux"], sp["q"], phys=sp["phys"], mthbc=sp["mthbc"],
                      regrid_interval=sp["regrid_interval"], rf=sp["refine"], hy=oracle.hydro(*sp["hydro"]))
        O.init()
        t0 = time.perf_counter()
        O.run(T, 1, 1.6, 0.9, 1.0, max_steps=4)
        s_o += time.perf_counter() - t0
        cu_o += O.cell_updates
    mxs = [sp["mx"] for sp in specs]
    return {
        "workload": f"{n} forests, mx in {{8,16,32}} ({mxs.count(8)}/{mxs.count(16)}/"
                    f"{mxs.count(32)}), levels 2-5, target patches log-uniform [50, 5000], "
                    f"{T:g} s simulated, regrid every 4 steps",
        "value": work / el_b, "unit": METRIC, "seconds": el_b,
        "one_by_one": {"value": work_s / el_s, "unit": METRIC, "seconds": el_s,
                       "note": "same forests, Forest.run one after another"},
        "speedup_vs_one_by_one": (work / el_b) / (work_s / el_s),
        "batch_equals_one_by_one": bool(same), "checked_forests": len(sample),
        "patches_initial": [int(min(patches0)), int(max(patches0)), int(sum(patches0))],
        "patches_max": [int(min(pmax)), int(max(pmax))],
        "rounds": bst["rounds"], "epochs": bst["epochs"], "regrids": bst["regrids"],
        "launches": bst["launches"], "cell_updates": work,
        "host_seconds": {"rounds": bst["s_rounds"], "regrid": bst["s_regrid"],
                         "epoch": bst["s_epoch"]},
        "cpu_oracle": {"value": cu_o / s_o, "unit": METRIC, "seconds": s_o, "cores": os.cpu_count(),
                       "kind": "port",
                       "sample": f"forests {picks} (quartile and median size), 4 step attempts each; "
                                 "per cell-update, not the whole batch"},
    }


def fserved_leg(args, dev=0):
    """Served AMR forests (config 3 as a request stream): forests as in the
    batched leg (mx drawn from {8, 16, 32}, levels 2..5, target patches
    log-uniform [50, 2000], reservoir + inflow hydrograph, regrid every 4
    steps, a bounded simulated time) arrive as a Poisson stream at 80 % of
    the capacity measured in a saturated calibration pass, into the forest
    server running its request loop on its own thread. Reports throughput,
    p50/p99 latency (submit to done), the slowdown of a sample against its
    isolated latency, and that the sample's results equal the isolated runs
    bit for bit; the calibration forests also run through Forest.run one by
    one (the same work as the saturated pass)."""
    import geoflood_gb300 as gf
    from geoflood_gb300 import synth
    from geoflood_gb300.serve import ForestRequest, ForestServer, Hydrograph

    n = args.fserved_forests
    T = args.batch_time
    g = np.random.default_rng(SEED + 5)
    targets = np.exp(g.uniform(np.log(50), np.log(2000), n))
    specs = [synth.flood_forest(SEED + 300 + k, float(targets[k])) for k in range(n)]

    def req(sp):
        h = sp["hydro"]
        return ForestRequest(mx=sp["mx"], nbx=sp["nbx"], nby=sp["nby"], minlevel=sp["minlevel"],
                             maxlevel=sp["maxlevel"], dx0=sp["dx0"], dy0=sp["dy0"], t_final=T,
                             aux=sp["aux"], q=sp["q"], mthbc=sp["mthbc"],
                             regrid_interval=sp["regrid_interval"], refine=sp["refine"],
                             phys=sp["phys"], nout=1, initial_dt=1.6,
                             hydro=Hydrograph(np.array(h[0]), np.array(h[1]), tuple(h[2]), h[3],
                                              h[4], h[5]))

    lanes = {} if args.fserved_lane_cells is None else {"lane_cells": args.fserved_lane_cells}
    if args.fserved_reserve_sms is not None:
        lanes["reserve_sms"] = args.fserved_reserve_sms
    srv = ForestServer(device=dev, **lanes)
    srv.start()
    # -- calibration: a saturated batch, throughput until half of it is done
    ncal = min(16, n)
    st_a = srv.stats()
    t0 = srv.clock()
    cal = [srv.submit(req(specs[k])) for k in range(ncal)]
    samples = []
    while True:
        st = srv.stats()
        samples.append((srv.clock(), st["cell_updates"] - st_a["cell_updates"], st["active"] + st["queued"]))
        if st["active"] + st["queued"] == 0:
            break
        time.sleep(0.002)
    half = next((t, w) for t, w, left in samples if left <= ncal // 2)
    cap = half[1] / max(half[0] - t0, 1e-9)
    cal_info = [srv.wait(i, timeout=600) for i in cal]
    for i in cal:
        srv.release(i)
    est_work = float(np.mean([i["cell_updates"] for i in cal_info]))
    sat_work = sum(i["cell_updates"] for i in cal_info)
    sat_s = max(i["t_done"] for i in cal_info) - t0
    order = np.argsort(targets)
    sample = sorted({int(order[int(round(f * (n - 1)))]) for f in np.linspace(0.0, 1.0, 12)})
    reqs = [req(sp).prepare() for sp in specs]   # raster blocks built before the stream

    def stream(rate, seed):
        """Poisson arrivals at `rate` forests/s; every forest waited for."""
        gaps = np.random.default_rng(seed).exponential(1.0 / rate, n)
        arrivals = np.cumsum(gaps) - gaps[0]
        st0 = srv.stats()
        t_start = srv.clock()
        ids, late = {}, 0
        for k in range(n):
            t_arr = t_start + arrivals[k]
            while srv.clock() < t_arr:
                time.sleep(min(0.002, max(t_arr - srv.clock(), 0.0)))
            late += srv.clock() - t_arr > 0.01
            ids[k] = srv.submit(reqs[k])
        infos = {k: srv.wait(ids[k], timeout=3600) for k in range(n)}
        outs = {k: srv.download(ids[k]) for k in sample if infos[k]["state"] == "done"}
        for k in range(n):
            srv.release(ids[k])
        st1 = srv.stats()
        t_end = max(i["t_done"] for i in infos.values())
        lat = np.array([i["t_done"] - i["t_submit"] for i in infos.values()])
        work = sum(i["cell_updates"] for i in infos.values())
        return {"infos": infos, "outs": outs, "late": late, "t_start": t_start, "t_end": t_end,
                "lat": lat, "work": work, "st0": st0, "st1": st1, "rate": rate,
                "failed": sum(1 for i in infos.values() if i["state"] != "done")}

    rate = args.fserved_rate or 0.8 * cap / est_work
    main_run = stream(rate, SEED + 6)
    low_run = stream(0.5 * cap / est_work, SEED + 7)
    # -- isolated re-runs of the sample: latency alone, same bits as in both streams
    iso = {}
    same = True
    for k in sample:
        sid = srv.submit(reqs[k])
        ik = srv.wait(sid, timeout=600)
        p, q, _ = srv.download(sid)
        srv.release(sid)
        iso[k] = ik
        for run in (main_run, low_run):
            o = run["outs"].get(k)
            same &= (o is not None and np.array_equal(p, o[0]) and np.array_equal(q, o[1])
                     and ik["steps"] == run["infos"][k]["steps"])

    def slowdowns(run):
        sl = [(run["infos"][k]["t_done"] - run["infos"][k]["t_submit"])
              / (iso[k]["t_done"] - iso[k]["t_submit"]) for k in sample]
        return {"p50": float(np.percentile(sl, 50)), "p99": float(np.percentile(sl, 99)),
                "max": float(max(sl)), "sample": len(sample)}

    detail = [{"mx": specs[k]["mx"], "npatch_max": iso[k]["npatch_max"], "steps": iso[k]["steps"],
               "isolated_s": iso[k]["t_done"] - iso[k]["t_submit"],
               "mixed_s": main_run["infos"][k]["t_done"] - main_run["infos"][k]["t_submit"],
               "mixed_50pct_s": low_run["infos"][k]["t_done"] - low_run["infos"][k]["t_submit"],
               "lane": iso[k]["lane"]} for k in sample]
    infos, lat, work = main_run["infos"], main_run["lat"], main_run["work"]
    t_start, t_end, late, failed = main_run["t_start"], main_run["t_end"], main_run["late"], main_run["failed"]
    st0, st1 = main_run["st0"], main_run["st1"]
    slow = slowdowns(main_run)
    slow["detail"] = detail
    srv.stop()
    srv.close()
    # -- the calibration forests through Forest.run, one after another
    ctx = gf.Context(dev)
    w1, s1 = 0, 0.0
    for k in range(ncal):
        sp = specs[k]
        ctx.set_phys(1, sp["phys"])
        F = gf.Forest(ctx, sp["mx"], sp["nbx"], sp["nby"], sp["minlevel"], sp["maxlevel"], sp["dx0"],
                      sp["dy0"], sp["aux"], sp["q"], mthbc=sp["mthbc"],
                      regrid_interval=sp["regrid_interval"], refine=sp["refine"], phys_slot=1)
        F.set_hydrograph(*sp["hydro"])
        tp = time.perf_counter()
        F.init()
        w1 += F.run(T, 1, 1.6, 0.9, 1.0)["cell_updates"]
        s1 += time.perf_counter() - tp
        F.close()
    ctx.close()
    mxs = [sp["mx"] for sp in specs]
    served_rate = work / (t_end - t_start)
    return {
        "workload": f"{n} forests, mx in {{8,16,32}} ({mxs.count(8)}/{mxs.count(16)}/{mxs.count(32)}), "
                    f"levels 2-5, target patches log-uniform [50, 2000], {T:g} s simulated, regrid "
                    "every 4 steps; Poisson arrivals at 80 % of the calibrated capacity",
        "value": served_rate, "unit": METRIC, "forests": n, "failed": failed,
        "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
        "slowdown_vs_isolated": slow,
        "alone_equals_mix": bool(same),
        "at_50pct_load": {"value": low_run["work"] / (low_run["t_end"] - low_run["t_start"]), "unit": METRIC,
                          "arrival_rate_per_s": low_run["rate"],
                          "p50_latency_s": float(np.percentile(low_run["lat"], 50)),
                          "p99_latency_s": float(np.percentile(low_run["lat"], 99)),
                          "slowdown_vs_isolated": slowdowns(low_run), "failed": low_run["failed"]},
        "saturated": {"value": sat_work / sat_s, "unit": METRIC, "forests": ncal, "seconds": sat_s,
                      "note": "the first forests of the stream submitted at once, until all are done"},
        "one_by_one": {"value": w1 / s1, "unit": METRIC, "seconds": s1,
                       "note": "the same forests through Forest.run (init included), one after another"},
        "saturated_vs_one_by_one": (sat_work / sat_s) / (w1 / s1),
        "capacity": {"value": cap, "unit": METRIC, "forests": ncal, "window_s": half[0] - t0,
                     "note": "saturated, until half of the forests are done; sets the arrival rate"},
        "arrival_rate_per_s": rate, "late_submissions": int(late), "stream_seconds": t_end - t_start,
        "cell_updates": work, "iterations": st1["iterations"] - st0["iterations"],
        "epochs": st1["epochs"] - st0["epochs"], "rounds": st1["rounds"] - st0["rounds"],
        "launches": st1["launches"] - st0["launches"], "regrids": st1["regrids"] - st0["regrids"],
        "host_seconds": {k: st1[k] - st0[k] for k in ("s_admit", "s_epoch", "s_rounds", "s_regrid")},
        "peak_device_bytes": st1["bytes_peak"],
    }


def large_leg(args, dev=0):
    """Large single scenario (config 5) as one forest: 2 x 2 brick, mx 32,
    levels 3..7 (2 m finest cells, 8192^2 equivalent), fractal DEM with a
    dendritic channel network, two-class Manning field (variable friction),
    inundated start (~17k finest patches), inflow on two sides, regrid every
    4 steps; a bounded number of step attempts of the 6 h run."""
    import geoflood_gb300 as gf
    from geoflood_gb300 import synth

    t0 = time.perf_counter()
    sp = synth.large_scenario()
    t_gen = time.perf_counter() - t0
    ctx = gf.Context(dev)
    ctx.set_phys(0, sp["phys"])
    F = gf.Forest(ctx, sp["mx"], sp["nbx"], sp["nby"], sp["minlevel"], sp["maxlevel"], sp["dx0"],
                  sp["dy0"], sp["aux"], sp["q"], mthbc=sp["mthbc"],
                  regrid_interval=sp["regrid_interval"], refine=sp["refine"])
    F.set_hydrograph(*sp["hydro"])
    t0 = time.perf_counter()
    F.init()
    t_init = time.perf_counter() - t0
    p0 = F.npatch
    lv = F.patches()[:, 0]
    t0 = time.perf_counter()
    st = F.run(21600.0, 1, 1.0, 0.9, 1.0, max_steps=args.large_steps)
    el = time.perf_counter() - t0
    F.close()
    ctx.close()
    # the oracle's forest driver on the same scenario, 2 step attempts (no
    # regrid falls inside them)
    import oracle
    from oracle import forest as of
    O = of.Forest(sp["mx"], sp["nbx"], sp["nby"], sp["minlevel"], sp["maxlevel"], sp["dx0"], sp["dy0"],
                  sp["aux"], sp["q"], phys=sp["phys"], mthbc=sp["mthbc"], regrid_interval=0,
                  rf=sp["refine"], hy=oracle.hydro(*sp["hydro"]))
    del sp
    O.init()
    t0 = time.perf_counter()
    O.run(21600.0, 1, 1.0, 0.9, 1.0, max_steps=2)
    s_o = time.perf_counter() - t0
    cu_o = O.cell_updates
    del O
    return {
        "workload": "large scenario: 2x2 brick, mx 32, levels 3-7 (8192^2 at 2 m), fractal DEM "
                    "Hurst 0.85 relief 50 m + dendritic channels, n 0.03/0.07 field, "
                    f"inundated start, {args.large_steps} step attempts, regrid every 4",
        "value": st["cell_updates"] / el, "unit": METRIC, "seconds": el,
        "steps": st["steps"], "rejects": st["rejects"], "regrids": st["regrids"],
        "simulated_s": st["t"], "patches_initial": int(p0), "patches_max": st["npatch_max"],
        "finest_patches_initial": int((lv == lv.max()).sum()),
        "cells_initial": int(p0) * 32 * 32,
        "seconds_generate": t_gen, "seconds_init": t_init,
        "cpu_oracle": {"value": cu_o / s_o, "unit": METRIC, "seconds": s_o, "cores": os.cpu_count(),
                       "kind": "port", "sample": "2 step attempts of the same scenario (per cell-update)"},
    }


def fp64_rates():
    """Measured FP64 pipe rates of this GPU (gf_measure_fp64_rates), ops/s."""
    import ctypes as C

    from geoflood_gb300 import _lib

    lib = _lib.load()
    r = (C.c_double * 4)()
    if lib.gf_measure_fp64_rates(int(os.environ.get("LOCAL_RANK", "0")), r) != 0:
        return None
    return {"dfma": r[0], "ddiv": r[1], "dsqrt": r[2], "ffma": r[3]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--served-only", action="store_true")
    ap.add_argument("--no-forest", action="store_true")
    ap.add_argument("--forest-only", action="store_true")
    ap.add_argument("--forest-steps", type=int, default=200)
    ap.add_argument("--batch-forests", type=int, default=64)
    ap.add_argument("--batch-time", type=float, default=10.0)
    ap.add_argument("--batched-only", action="store_true")
    ap.add_argument("--fserved-forests", type=int, default=32)
    ap.add_argument("--fserved-only", action="store_true")
    ap.add_argument("--fserved-lane-cells", type=int, default=None,
                    help="forest server: small-lane threshold in cells (0: one lane)")
    ap.add_argument("--fserved-reserve-sms", type=int, default=None)
    ap.add_argument("--fserved-rate", type=float, default=None,
                    help="forest arrivals per second (default: 80 %% of the calibrated capacity)")
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tiles", default="",
                    help="pin tile variants instead of autotuning: mx:throughput:latency,... "
                         "(e.g. 32:3:7)")
    ap.add_argument("--large-only", action="store_true")
    ap.add_argument("--large-steps", type=int, default=24)
    ap.add_argument("--no-dem", action="store_true")
    ap.add_argument("--dem-only", action="store_true")
    ap.add_argument("--served-scenarios", type=int, default=16)
    ap.add_argument("--served-time-scale", type=float, default=1.0,
                    help="multiplies every scenario time (horizon, hydrograph rise)")
    ap.add_argument("--served-cal-seconds", type=float, default=8.0)
    ap.add_argument("--served-sample", type=int, default=6,
                    help="scenarios re-run alone for the slowdown (size-stratified)")
    ap.add_argument("--served-rate", type=float, default=None,
                    help="served stream: arrivals per second (default: 80 %% of the measured capacity)")
    ap.add_argument("--served-no-split", action="store_true",
                    help="served stream: one round queue per lane (patch sizes as graph branches)")
    ap.add_argument("--served-no-cull", action="store_true",
                    help="update every patch of every served scenario every step")
    ap.add_argument("--served-low-load", action="store_true",
                    help="also run the first half of the stream at 50 %% load")
    ap.add_argument("--detail", default=None,
                    help="write every figure of the run (per-leg detail) to this JSON file")
    ap.add_argument("--served-reserve-sms", type=int, default=None)
    ap.add_argument("--served-lanes", default="1e5,1e6",
                    help="cell-count boundaries between the server's size lanes")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.large_only:
        print(json.dumps({"large": large_leg(args)}))
        return 0
    if args.dem_only:
        print(json.dumps({"dem": dem_leg(args)}))
        return 0
    if args.fserved_only:
        print(json.dumps({"served_amr": fserved_leg(args)}))
        return 0
    if args.batched_only:
        print(json.dumps({"batched": batched_leg(args)}))
        return 0
    if args.forest_only:
        print(json.dumps({"forest": forest_leg(args)}))
        return 0
    if args.served_only:
        print(json.dumps({"served": served_stream(args)}))
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
