#!/usr/bin/env python3
"""Benchmark of the GB300 hydro path: FP64 cell-updates/s.

Default workload (the single large instance): bi-material Sod along Y on a
2048x2048 mesh over [0,1]^2, a 50/50 mixed cell row at the interface, VNR
Lagrange scheme, order-2 remap, Superbee limiter with PenteBorne (pure),
A1 dual mass flux, 200 cycles, FP64.  One "step" is one full cycle
(Lagrange + two directional remap sweeps + dual remap + remap final) over
all 4,194,304 cells.  The state (~1.9 GB) is far larger than L2, so every
cycle streams it from HBM.

  value      device time (CUDA events on the run's stream) of K cycles,
             state resident in HBM
  e2e        the same work through the C ABI with host buffers: run
             creation from the options (the initial state is built on the
             device; the host uploads the 128-byte control block), K cycles,
             fetch of the final fields (device->host)
  roofline   the dominant kernel's algorithmic bytes / measured launch time
             against the measured HBM copy bandwidth, plus its FP64 rate
             against the measured FP64 FMA throughput (the kernels are FP64
             instruction bound on GB300)
  cpu_baseline  the C restatement of the reference (oracle/port, OpenMP on
             all host cores) on a bounded sample of the same workload

  --impl reference   times the reference's CPU algorithm (the C restatement;
                     the reference's own build cannot exist on this host) on
                     the same workload, on all host cores.
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

ROOT = Path(__file__).resolve().parent
CTRL_BYTES = 128  # the run's control block, the one host->device copy of creation
sys.path.insert(0, str(ROOT))

METRIC = "FP64 cell-updates/s on 1 GB300 batched/served vs plain GPU vs CPU; p50/p99"
UNIT = "cell-updates/s"


def workload_spec(M, n: int = 2048, cycles: int = 200):
    s = M.default_spec()
    s.scheme, s.test_case, s.nbmat = M.SCHEME_VNR, 16, 2  # BiSodCaseY
    s.nx = s.ny = n
    s.dx = s.dy = 1.0 / n
    s.final_time, s.output_time, s.dt_init, s.dt_min = 0.2, 1e-2, 1e-4, 1e-12
    s.space_order, s.projection, s.projection_order = 2, 1, 2
    s.limiter = M.LIMITERS["superBee"]
    s.pb, s.pb_mixte = 1, 0
    s.limiter_pure, s.pb_complet = M.LIMITERS["arithmeticG"], 0
    s.pseudo_centree, s.dual_mass_flux = 0, 0
    s.init_variant = 1
    s.max_cycles = cycles
    return s


WORKLOAD = {
    "workload": "bi-material Sod Y, 2048x2048 cells, 50/50 mixed interface row, "
                "VNR + order-2 remap, superBee + PenteBorne pure, A1 dual flux, "
                "200 cycles",
    "mesh": [2048, 2048], "nbmat": 2, "cycles": 200, "scheme": "VNR",
    "projection_order": 2, "limiter": "superBee", "pente_borne": "pure",
    "dual_mass_flux": "A1", "state_bytes": None,
    "l2": "state (~1.9 GB) >> L2 (129 MB): every cycle streams it from HBM",
}


# Algorithmic (compulsory) bytes per unit of each kernel: every input plane
# read once, every output plane written once; units are cells or nodes.
def algorithmic_bytes(kind: str, nb: int, pb: bool) -> int:
    nc = 3 * nb + 1
    d = 8
    table = {
        "k_lag_nodes": 18,                       # u, cell mass, p, q, cqs / u, XL, m
        "k_lag_cells": (7 + 7 * nb) + (8 + nb + 2 * nc),
        "k_sweep_grad": (nc + 3 + (4 if pb else 0)) + (2 * nc if pb else nc),
        "k_sweep_face": (2 * nc if pb else 2 * nc + 2) + nc,
        "k_sweep_update": (2 * nc + 5) + (nc + 2 * nb) + (nc + 1) // 2,
        "k_dual_grad": 5,
        "k_dual_update": (2 * nb + 2 + 8) + 5,
        "k_final": (nc + 2) + (6 + 7 * nb + 1),
    }
    return table.get(kind, 0) * d


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


class Clocks:
    """Samples nvidia-smi clocks / throttle reasons while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self) -> dict:
        self.f.flush()
        rows = []
        for line in Path(self.f.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[k] for _, _, r in rows for k in range(4)
                          if r[k].lower() in ("active", "1")})
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def barrier_max(value: float, world: int) -> float:
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(spec_fn, budget_s: float = 25.0) -> dict:
    """The C restatement on all host cores, a bounded sample of the workload:
    the full 2048^2 mesh, whole cycles until ~budget_s of CPU time."""
    from oracle import port
    cores = port.num_threads()
    spec = spec_fn()
    run = port.PortRun(spec)
    run.step(1)  # warm: first touch of every array
    n, t0 = 0, time.perf_counter()
    while True:
        run.step(1)
        n += 1
        el = time.perf_counter() - t0
        if el > budget_s or n >= 50:
            break
    cells = spec.nx * spec.ny
    run.close()
    return {"value": cells * n / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} cycles of the 2048x2048 workload (cycles 2..{n + 1}) "
                      f"on {cores} OpenMP threads, {el:.1f} s"}


def run_reference(args) -> None:
    rank, world, _ = dist_env()
    if rank != 0:
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    import mahyco_gb300 as M
    from oracle import port
    spec = workload_spec(M, 2048, 200)
    cores = port.num_threads()
    run = port.PortRun(spec)
    for _ in range(min(args.warmup, 1)):
        run.step(1)
    budget = 150.0
    n, t0 = 0, time.perf_counter()
    while n < args.steps:
        run.step(1)
        n += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    val = spec.nx * spec.ny * n / el
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT,
        "n_gpus": args.gpus, "steps": n, "warmup": min(args.warmup, 1),
        "ms_per_step": 1e3 * el / n, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(WORKLOAD, form="cpu"),
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{n} cycles of the 2048x2048 workload on "
                                   f"{cores} OpenMP threads (time-capped at "
                                   f"{budget:.0f} s)"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


BATCH_WORKLOAD = {
    "workload": "512 independent VNR runs, order-2 remap, minmod or superBee, "
                "no PenteBorne: 1/3 Sod (X or Y, 1 or 2 materials), 1/3 Sedov, "
                "1/3 advection step; nx log-uniform 64..1024, ny 64..256 "
                "(std::mt19937_64 seed 20261203), 100 cycles each",
    "instances": 512, "seed": 20261203,
    "l2": "state (~20 GB) >> L2 (129 MB)",
}


def bench_batch(M, ctx, args, local: int) -> dict:
    """The mixed batch: plain path (each run through its own CUDA graph, one
    after another) against the batched path (one persistent launch per phase
    for all 512 runs), on the same runs at nearby cycles."""
    from mahyco_gb300.workloads import batch_mix
    mix = batch_mix(args.batch_n)
    cells = sum(i.cells for i in mix)
    t0 = time.perf_counter()
    runs = [M.Run(i.spec(M), ctx) for i in mix]
    create_s = time.perf_counter() - t0
    state = sum(r.device_bytes for r in runs)
    import ctypes
    lib = M.lib()
    stream = ctypes.c_void_p(ctx.stream)
    # plain path: warm (graph capture) then K2 cycles of every run, enqueued
    # back to back, timed with events on the context's stream
    K2 = 8
    for r in runs:
        r.enqueue(1)
    for r in runs:
        r.sync()
    import torch
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ext = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    launches0 = sum(r.kernel_launches for r in runs)
    with Clocks(local) as clk_plain:
        ev0.record(ext)
        for r in runs:
            r.enqueue(K2)
        ev1.record(ext)
        ev1.synchronize()
    plain_ms = ev0.elapsed_time(ev1)
    plain_launches = sum(r.kernel_launches for r in runs) - launches0
    plain_val = cells * K2 / (plain_ms * 1e-3)
    # batched path: tuning cycles + warm-up, then K timed cycles
    batch = M.Batch(runs, ctx)
    batch.step(11 + 3)  # 11 tuning cycles (10 candidates + warm-up), 3 warm
    K = args.batch_steps
    b0 = batch.kernel_launches
    with Clocks(local) as clk_batch:
        bms = batch.timed(K)
    b_launches = batch.kernel_launches - b0
    bval = cells * K / (bms * 1e-3)
    prof = batch.profile(2)
    kinds = {k: v for k, v in prof.items() if v[1] > 0}
    t1 = time.perf_counter()
    left = batch.step(100)
    fetched = sum(r.fetch("density").nbytes for r in runs)
    finish_s = time.perf_counter() - t1
    cyc = [r.time()[2] for r in runs]
    errs = sum(1 for r in runs if r.error()[0] & ~M.ERR_NEGATIVE)
    cfg = batch.config()
    for r in runs:
        r.close()
    return {
        "value": bval, "unit": UNIT, "ms_per_step": bms / K, "steps": K,
        "gpu_launches": b_launches,
        "plain_mix": {"value": plain_val, "unit": UNIT, "ms_per_step": plain_ms / K2,
                      "steps": K2, "gpu_launches": plain_launches,
                      "clocks": clk_plain.summary(),
                      "how": "each run's own CUDA graph (8 cycles), runs enqueued "
                             "one after another, events around the sweep"},
        "speedup_vs_plain_mix": bval / plain_val,
        "cells": cells, "state_bytes": state, "create_s": create_s,
        "finish_s": finish_s, "fetch_bytes": fetched, "runs_left": left,
        "cycles_done": [min(cyc), max(cyc)], "runs_in_error": errs,
        "tuning": cfg, "clocks": clk_batch.summary(),
        "kernel_ms": {k: [round(v[0], 4), v[1]] for k, v in kinds.items()},
        "config": BATCH_WORKLOAD,
    }


SERVE_WORKLOAD = {
    "workload": "Poisson request streams; each request one VNR run drawn like the "
                "batch mix (Sod / Sedov / advection, order-2 remap, minmod or "
                "superBee) with nx, ny log-uniform 32..2048, 1-3 materials, "
                "50-500 cycles (std::mt19937_64 seed 7 + rate); admission against a "
                "150 GB HBM budget, runs resident until they end",
    "budget_bytes": 150 * 10**9,
}


def bench_serve(M, args, local: int) -> dict:
    """Continuous batching under Poisson arrivals: per rate, n requests are
    submitted at their arrival times; latency is submission -> retirement;
    throughput is the cell-updates of all requests over first arrival ->
    last retirement."""
    from mahyco_gb300.workloads import request_stream
    rates = [float(x) for x in args.serve_rates.split(",") if x]
    out = []
    for lam in rates:
        reqs = request_stream(lam, args.serve_n)
        ctx = M.Context(local)
        srv = M.Server(ctx, budget=SERVE_WORKLOAD["budget_bytes"], tick_cycles=8,
                       prep_threads=8)
        lat = []
        t0 = time.perf_counter()
        with Clocks(local) as clk:
            for r in reqs:
                dt = r.arrival - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                srv.submit(r.inst.spec(M))
                while (d := srv.poll(0.0)) is not None:
                    lat.append(d)
            while len(lat) < len(reqs):
                d = srv.poll(5.0)
                if d is not None:
                    lat.append(d)
                if time.perf_counter() - t0 > args.serve_timeout:
                    break
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.stop(drain=False)
        ctx.close()
        ls = sorted(d.latency_s for d in lat)
        work = sum(d.cells * d.cycles for d in lat)

        def pct(q):
            return ls[min(len(ls) - 1, int(q * len(ls)))] if ls else None
        out.append({
            "rate_req_s": lam, "requests": len(reqs), "completed": len(lat),
            "failed": sum(1 for d in lat if d.status < 0),
            "p50_latency_s": pct(0.50), "p99_latency_s": pct(0.99),
            "cell_updates": work, "wall_s": wall,
            "value": work / wall if wall > 0 else None, "unit": UNIT,
            "peak_resident": st["peak_resident"], "peak_bytes": st["peak_bytes"],
            "ticks": st["ticks"], "clocks": clk.summary(),
        })
    return {"rates": out, "config": SERVE_WORKLOAD,
            "value": max((o["value"] or 0) for o in out) if out else None, "unit": UNIT}


def triple_point_spec(M, nx: int = 1792, ny: int = 768, cycles: int = 300,
                      order: int = 3, pb: int = 0):
    """Three-material triple point on [0,7]x[0,3]: Eucclhyd, superBee,
    CFL 0.4, exponents 1.5 / 1.4 / 1.5, regions x <= 1 and y <= 1.5."""
    s = M.default_spec()
    s.scheme, s.test_case, s.nbmat = M.SCHEME_EUCCLHYD, 13, 3
    s.nx, s.ny = nx, ny
    s.dx, s.dy = 7.0 / nx, 3.0 / ny
    for m, g in enumerate((1.5, 1.4, 1.5)):
        s.eos[m] = 101
        s.gamma[m] = g
    s.gamma_scalar, s.cfl = 1.4, 0.4
    s.final_time, s.dt_min, s.space_order = 100.0, 1e-12, 2
    s.projection, s.projection_order = 1, order
    s.limiter = M.LIMITERS["superBee"]
    s.pb, s.pb_mixte, s.limiter_pure, s.pb_complet = pb, pb, M.LIMITERS["arithmeticG"], 0
    s.init_variant = 3
    s.max_cycles = cycles
    return s


EUC_WORKLOAD = {
    "workload": "triple point, 3 materials, 1792x768 cells on [0,7]x[0,3], "
                "Eucclhyd + order-3 remap, superBee, CFL 0.4, gamma 1.5/1.4/1.5",
    "mesh": [1792, 768], "nbmat": 3, "scheme": "Eucclhyd", "projection_order": 3,
    "limiter": "superBee", "pente_borne": "non",
    "note": "with PenteBorne mixte and order 3 the reference itself stops in "
            "cycle 2 (negative, then NaN densities: it takes the order-3 face "
            "value as an integrated flux); this path reproduces that and stops "
            "the same way (see configured_variant), so the throughput is "
            "measured on the same case without PenteBorne",
}


def bench_euc(M, ctx, args, local: int) -> dict:
    """Eucclhyd on the triple point: device time of K cycles (state resident),
    per-kernel times, the configured PenteBorne variant's outcome, and the
    C restatement on a bounded sample."""
    K = args.euc_steps
    w = M.Run(triple_point_spec(M, cycles=args.warmup + 1), ctx)
    w.timed(args.warmup)
    w.close()
    run = M.Run(triple_point_spec(M, cycles=K + 8), ctx)
    cells = 1792 * 768
    l0 = run.kernel_launches
    with Clocks(local) as clk:
        ms = run.timed(K)
    launches = run.kernel_launches - l0
    prof = run.profile(4)
    err = run.error()[0]
    run.close()
    kinds = {k: v for k, v in prof.items() if v[1] > 0}
    cfg_run = M.Run(triple_point_spec(M, cycles=10, pb=1), ctx)
    cfg_run.simulate()
    code, cell = cfg_run.error()
    configured = {"pente_borne": "mixte", "cycles_done": cfg_run.time()[2],
                  "error_word": code, "error_cell": cell,
                  "reference_behaviour": "cell--Nan 2, exit(1) in cycle 2"}
    cfg_run.close()
    out = {"value": cells * K / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / K,
           "steps": K, "gpu_launches": launches, "error_word": err,
           "clocks": clk.summary(), "config": EUC_WORKLOAD,
           "configured_variant": configured,
           "kernel_ms": {k: [round(v[0], 4), v[1]] for k, v in kinds.items()}}
    if not args.no_cpu:
        from oracle import port
        pr = port.PortRun(triple_point_spec(M, cycles=1000))
        pr.step(1)
        n, t0 = 0, time.perf_counter()
        while n < 20 and time.perf_counter() - t0 < 15.0:
            pr.step(1)
            n += 1
        el = time.perf_counter() - t0
        pr.close()
        out["cpu_baseline"] = {"value": cells * n / el, "unit": UNIT,
                               "cores": port.num_threads(), "kind": "port",
                               "sample": f"{n} cycles of the 1792x768 triple point "
                                         f"on {port.num_threads()} OpenMP threads, "
                                         f"{el:.1f} s"}
    return out


def run_ours(args) -> None:
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    import mahyco_gb300 as M
    ctx = M.Context(local)
    W, K = args.warmup, args.steps
    n = args.mesh
    spec = workload_spec(M, n, K + 16)
    cells = n * n
    # warm-up: graph instantiation, first launches, clocks up
    w = M.Run(workload_spec(M, n, W + 1), ctx)
    w.timed(W)
    w.close()
    run = M.Run(spec, ctx)
    state_bytes = run.device_bytes
    launches0 = run.kernel_launches
    barrier_max(0.0, world)
    with Clocks(local) as clk:
        ms = run.timed(K)
    clocks = clk.summary()
    launches = run.kernel_launches - launches0
    ms = barrier_max(ms, world)
    value = cells * K * world / (ms * 1e-3)
    # per-kernel profile over 8 further cycles of the same run
    prof = run.profile(8)
    run.close()
    # dominant kernel and its roofline
    kinds = {k: v for k, v in prof.items() if v[1] > 0}
    dom = max(kinds, key=lambda k: kinds[k][0])
    dom_ms, dom_n = kinds[dom]
    per_launch_ms = dom_ms / dom_n
    node_kernel = dom in ("k_lag_nodes", "k_dual_grad", "k_dual_update")
    units = (n + 1) * (n + 1) if node_kernel else cells
    alg = algorithmic_bytes(dom, spec.nbmat, bool(spec.pb)) * units
    achieved = alg / (per_launch_ms * 1e-3) / 1e9
    peaks = load_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    prof_file = ROOT / "profiles" / "kernel_counters_bisod_vnr.json"
    traffic = None
    fp64 = None
    fp64_peak = M.fp64_peak_tflops(local)
    if prof_file.exists():
        pj = json.loads(prof_file.read_text())
        kp = pj.get("kernels", {}).get(dom, {})
        if "dram_bytes_per_unit" in kp:
            traffic = kp["dram_bytes_per_unit"] * units
        if "fp64_flops_per_unit" in kp:
            fl = kp["fp64_flops_per_unit"] * units
            ach = fl / (per_launch_ms * 1e-3) / 1e12
            fp64 = {"achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                    "frac": ach / fp64_peak, "flops_per_launch": fl,
                    "peak_source": "measured DFMA chain (hydro_fp64_peak)"}
    if fp64 is None:
        fp64 = {"achieved": None, "peak": fp64_peak, "unit": "TFLOP/s",
                "peak_source": "measured DFMA chain (hydro_fp64_peak)"}
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm,
                "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
                "algorithmic_bytes_per_launch": alg,
                "launch_ms": per_launch_ms,
                "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)"
                if not peaks.get("fallback") else "of fallback",
                "fp64": fp64}
    # end to end through the C ABI with host buffers
    t0 = time.perf_counter()
    e = M.Run(workload_spec(M, n, K), ctx)
    e.step(K)
    outs = [e.fetch(f) for f in ("density", "pressure", "energy", "fracvol_env",
                                 "node_velocity")]
    e2e_s = time.perf_counter() - t0
    h2d = CTRL_BYTES  # the control block; the initial state is built on the device
    d2h = sum(o.nbytes for o in outs)
    e.close()
    e2e = {"value": cells * K / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(h2d / K), "d2h_bytes_per_step": int(d2h / K),
           "includes": "run creation (device-built initial state), K cycles, fetch of 5 fields"}
    if rank != 0:
        return
    cpu = None if args.no_cpu else cpu_baseline(lambda: workload_spec(M, n, 200))
    cfg = dict(WORKLOAD, form="plain", state_bytes=state_bytes)
    if n != 2048:
        cfg["mesh"] = [n, n]
        cfg["workload"] = cfg["workload"].replace("2048x2048", f"{n}x{n}")
    batched = None if args.no_batch else bench_batch(M, ctx, args, local)
    served = None if args.no_serve else bench_serve(M, args, local)
    eucclhyd = None if args.no_euc else bench_euc(M, ctx, args, local)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": ms / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (analytic initial state)", "config": cfg,
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
        "gpu_launches": launches,
        "kernel_ms": {k: [round(v[0], 4), v[1]] for k, v in kinds.items()},
        "batched": batched,
        "served": served,
        "eucclhyd": eucclhyd,
    }
    print(json.dumps(line))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mesh", type=int, default=2048)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-n", type=int, default=512)
    ap.add_argument("--batch-steps", type=int, default=40)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-euc", action="store_true")
    ap.add_argument("--euc-steps", type=int, default=60)
    ap.add_argument("--serve-rates", default="50,200,1000,2000")
    ap.add_argument("--serve-n", type=int, default=24)
    ap.add_argument("--serve-timeout", type=float, default=120.0)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
