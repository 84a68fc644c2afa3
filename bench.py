#!/usr/bin/env python3
"""Benchmark of the GB300 hydro path: FP64 cell-updates/s.

Default workload (the single large instance): bi-material Sod along Y on a
2048x2048 mesh over [0,1]^2, a 50/50 mixed cell row at the interface, VNR
Lagrange scheme, order-2 remap, Superbee limiter with PenteBorne (pure),
A1 dual mass flux, 200 cycles, FP64.  One "step" is one full cycle
(Lagrange + two directional remap sweeps + dual remap + remap final) over
all 4,194,304 cells.  The state (~3.9 GB) is far larger than L2, so every
cycle streams it from HBM.

  value      device time (CUDA events on the run's stream) of the last K
             cycles of the configured 200-cycle window (cycles 200-K+1..200,
             the first 200-K advanced untimed), state resident in HBM
  e2e        the whole 200-cycle job through the C ABI with host buffers:
             run creation from the options (the initial state is built on
             the device; the host uploads the 128-byte control block), 200
             cycles, fetch of the final fields (device->host)
  developed  the same deck advanced untimed until most nodes move (the
             flow developed), then K cycles timed: the regime where the
             exact at-rest shortcuts are taken almost nowhere
  roofline   the dominant kernel's algorithmic bytes / measured launch time
             against the measured HBM copy bandwidth, plus its FP64 rate
             against the measured FP64 FMA throughput
  cpu_baseline  the C restatement of the reference (oracle/port, OpenMP on
             all host cores) on a bounded sample of the same workload
  summary    the headline figures of every record, last on the line

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

import numpy as np

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


CYCLES = 200  # the configured window of the large single instance


def timed_window(K: int, W: int) -> tuple[int, int]:
    """(untimed cycles before the timed ones, run length): the K timed
    cycles end the configured window; with K + W above it the window is
    extended so that W warm-up cycles still come first."""
    adv = CYCLES - K if K + W <= CYCLES else W
    return adv, max(CYCLES, adv + K)


def workload_config(K: int, W: int, n: int = 2048) -> dict:
    adv, length = timed_window(K, W)
    return {
        "workload": f"bi-material Sod Y, {n}x{n} cells, 50/50 mixed interface row, "
                    "VNR + order-2 remap, superBee + PenteBorne pure, A1 dual flux, "
                    f"{CYCLES} cycles",
        "mesh": [n, n], "nbmat": 2, "cycles": CYCLES, "scheme": "VNR",
        "projection_order": 2, "limiter": "superBee", "pente_borne": "pure",
        "dual_mass_flux": "A1",
        "l2": "state (~3.9 GB) >> L2 (129 MB): every cycle streams it from HBM",
    }


# Algorithmic (compulsory) bytes per unit of each kernel: every plane it
# must read read once, every plane it must write written once; units are
# cells or nodes (a face counts as a cell); nc live remap components, nb
# materials.  `rest`: the benchmark's regime, where almost every cell is at
# rest: the slope kernel only records that a cell's plateau-slope integrals
# are zeros (one flag byte) and the update reads the flags instead of those
# planes and stores only the components a sweep changed, so what such a cell
# must move is counted; otherwise (a developed flow) every plane.
def algorithmic_bytes(kind: str, nb: int, pb: bool, rest: bool = False) -> int:
    nc = 3 * nb + 1
    d = 8
    table = {
        # u, cell mass, p, q, corner normals / u, Lagrange position, node mass
        "k_lag_nodes": 18,
        # state planes in / Lagrange state, remap inputs (U, Phi), geometry out
        "k_lag_cells": (7 + 7 * nb) + (8 + nb + 2 * nc),
        # without PenteBorne: Phi, centroid in / nc face gradients out
        "k_face_grad": (nc + 1) + nc,
        # PenteBorne: Phi, centroid, width, 2 node velocities, 2 outer
        # normals in / the two plateau-slope integrals out; otherwise Phi,
        # nc face gradients, centroid, width, 2 node velocities in / nc
        # face values out
        "k_sweep_grad": (nc + 6) + 2 * nc if pb else (2 * nc + 4) + nc,
        # order 1 / order 3 face values
        "k_sweep_face": (2 * nc if pb else 2 * nc + 2) + nc,
        # U, the two integrals (PenteBorne) or the face values, 2 node
        # velocities, 2 outer normals in / U, the nodal mass-flux shares,
        # Phi and the flags in the first sweep (half of the launches) out
        "k_sweep_update": ((3 * nc + 4) if pb else (2 * nc + 5)) + (nc + nb) + (nc + 1) // 2,
        "k_dual_grad": 5,
        "k_dual_update": (2 * nb + 2 + 8) + 5,
        "k_final": (nc + 2) + (6 + 7 * nb + 1),
    }
    if rest:
        # a pure cell at rest leaves out the stores of the values it read
        # and found unchanged (divergence, sound speed, the root's argument,
        # its material's pseudo-viscosity), and, its Lagrange geometry planes
        # holding the rest geometry already (one flag byte in), the rest
        # geometry's four loads past the volume and the five stores
        table["k_lag_cells"] -= 4 + 4 + 5 - 0.125
    if rest and pb:
        # a cell at rest: the node velocity along the sweep in / its flag
        # byte out; U, 2 node velocities, 2 outer normals and the flag bytes
        # in / the mass-flux shares (and a flag byte) out
        table["k_sweep_grad"] = 1.25
        table["k_sweep_update"] = (nc + 4.25) + (nb + 0.125)
    return int(table.get(kind, 0) * d)


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
    """The reference's CPU algorithm (the C restatement, bit for bit the
    reference) on all host cores: W warm-up cycles, then K timed cycles of
    the same deck (time-capped)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    import mahyco_gb300 as M
    from oracle import port
    K, W = args.steps, args.warmup
    spec = workload_spec(M, args.mesh, CYCLES + K + W)
    cores = port.num_threads()
    run = port.PortRun(spec)
    run.step(W)
    budget = 150.0
    n, t0 = 0, time.perf_counter()
    while n < K:
        run.step(1)
        n += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    val = spec.nx * spec.ny * n / el
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT,
        "n_gpus": args.gpus, "steps": n, "warmup": W,
        "ms_per_step": 1e3 * el / n, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (analytic initial state)",
        "config": workload_config(K, W, args.mesh), "form": "cpu",
        "window": [W + 1, W + n],
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"cycles {W + 1}..{W + n} of the {args.mesh}x{args.mesh} "
                                   f"workload after {W} warm-up cycles, on {cores} OpenMP "
                                   f"threads (time-capped at {budget:.0f} s; the port does "
                                   "the reference's full arithmetic on every cell, its "
                                   "per-cycle cost barely depends on the cycle)"},
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
    for all 512 runs), each on its own copy of the same runs, timed over the
    same cycles (WARM untimed cycles first: the batch autotunes in 11 of
    them)."""
    from mahyco_gb300.workloads import batch_mix
    import torch
    mix = batch_mix(args.batch_n)
    cells = sum(i.cells for i in mix)
    K, WARM = args.batch_steps, 14
    # plain path: every run's own 8-cycle graph, runs enqueued back to back,
    # events on the context's stream around the K cycles of all of them
    plain_runs = [M.Run(i.spec(M), ctx) for i in mix]
    for r in plain_runs:
        r.enqueue(WARM)
    for r in plain_runs:
        r.sync()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ext = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    launches0 = sum(r.kernel_launches for r in plain_runs)
    with Clocks(local) as clk_plain:
        ev0.record(ext)
        for r in plain_runs:
            r.enqueue(K)
        ev1.record(ext)
        ev1.synchronize()
    plain_ms = ev0.elapsed_time(ev1)
    plain_launches = sum(r.kernel_launches for r in plain_runs) - launches0
    plain_val = cells * K / (plain_ms * 1e-3)
    plain_density = [r.fetch("density") for r in plain_runs[:8]]
    for r in plain_runs:
        r.close()
    # batched path on a fresh copy of the same runs
    t0 = time.perf_counter()
    runs = [M.Run(i.spec(M), ctx) for i in mix]
    create_s = time.perf_counter() - t0
    state = sum(r.device_bytes for r in runs)
    batch = M.Batch(runs, ctx)
    batch.step(WARM)  # 11 tuning cycles (10 candidates + warm-up), 3 warm
    b0 = batch.kernel_launches
    with Clocks(local) as clk_batch:
        bms = batch.timed(K)
    b_launches = batch.kernel_launches - b0
    bval = cells * K / (bms * 1e-3)
    same = all(np.array_equal(a, r.fetch("density")) for a, r in zip(plain_density, runs))
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
        "timed_cycles": [WARM + 1, WARM + K],
        "gpu_launches": b_launches,
        "plain_mix": {"value": plain_val, "unit": UNIT, "ms_per_step": plain_ms / K,
                      "steps": K, "timed_cycles": [WARM + 1, WARM + K],
                      "gpu_launches": plain_launches,
                      "clocks": clk_plain.summary(),
                      "how": "each run's own CUDA graph (8 cycles), runs enqueued "
                             "one after another, events around the K cycles of all"},
        "speedup_vs_plain_mix": bval / plain_val,
        "plain_equals_batched_at_window_end": same,
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
    submitted at their arrival times; latency is submission -> retirement,
    split into the admission wait (submission -> admission against the HBM
    budget and the slots) and the time resident on the device (placement ->
    retirement); throughput is the cell-updates of all requests over first
    arrival -> last retirement.  The first rate is below the server's
    capacity (about 7 requests/s of this mix), so its latencies are service
    times rather than queue drain."""
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
        work = sum(d.cells * d.cycles for d in lat)

        def pct(vals, q):
            vals = sorted(vals)
            return vals[min(len(vals) - 1, int(q * len(vals)))] if vals else None
        out.append({
            "rate_req_s": lam, "requests": len(reqs), "completed": len(lat),
            "failed": sum(1 for d in lat if d.status < 0),
            "p50_latency_s": pct([d.latency_s for d in lat], 0.50),
            "p99_latency_s": pct([d.latency_s for d in lat], 0.99),
            "p50_wait_s": pct([d.wait_s for d in lat], 0.50),
            "p99_wait_s": pct([d.wait_s for d in lat], 0.99),
            "p50_resident_s": pct([d.resident_s for d in lat], 0.50),
            "p99_resident_s": pct([d.resident_s for d in lat], 0.99),
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


def roofline_of(M, kinds: dict, spec, regime: str, local: int) -> dict:
    """Roofline of the dominant kernel of a per-kernel profile: algorithmic
    bytes per launch over its mean CUDA-event launch time against the
    measured HBM bandwidth; DRAM traffic and FP64 flops per unit from the
    committed ncu counters of the same regime ("kernels": the benchmark's
    early cycles, "developed": the developed flow), scaled by the units."""
    n = spec.nx
    cells = spec.nx * spec.ny
    dom = max(kinds, key=lambda k: kinds[k][0])
    dom_ms, dom_n = kinds[dom]
    per_launch_ms = dom_ms / dom_n
    node_kernel = dom in ("k_lag_nodes", "k_dual_grad", "k_dual_update")
    units = (n + 1) * (spec.ny + 1) if node_kernel else cells
    alg = algorithmic_bytes(dom, spec.nbmat, bool(spec.pb), rest=(regime == "kernels")) * units
    achieved = alg / (per_launch_ms * 1e-3) / 1e9
    peaks = load_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    prof_file = ROOT / "profiles" / "kernel_counters_bisod_vnr.json"
    traffic, fp64 = None, None
    fp64_peak = M.fp64_peak_tflops(local)
    if prof_file.exists():
        pj = json.loads(prof_file.read_text())
        table = pj.get(regime, {})
        table = table.get("kernels", table)
        kp = table.get(dom) or table.get(dom + "_pb") or table.get(dom + "_f", {})
        if "dram_bytes_per_unit" in kp:
            traffic = kp["dram_bytes_per_unit"] * units
        if "fp64_flops_per_unit" in kp:
            fl = kp["fp64_flops_per_unit"] * units
            ach = fl / (per_launch_ms * 1e-3) / 1e12
            fp64 = {"achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                    "frac": ach / fp64_peak, "flops_per_launch": fl,
                    "pipe_busy_pct_ncu": kp.get("fp64_pipe_pct"),
                    "peak_source": "measured DFMA chain (hydro_fp64_peak)"}
    if fp64 is None:
        fp64 = {"achieved": None, "peak": fp64_peak, "unit": "TFLOP/s",
                "peak_source": "measured DFMA chain (hydro_fp64_peak)"}
    return {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm,
            "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
            "algorithmic_bytes_per_launch": alg, "launch_ms": per_launch_ms,
            "counters": f"profiles/kernel_counters_bisod_vnr.json [{regime}]",
            "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)"
            if not peaks.get("fallback") else "of fallback",
            "fp64": fp64}


def path_traffic(kinds: dict, spec, regime: str, ms_per_cycle: float) -> dict | None:
    """Whole-cycle DRAM bytes per cell from the committed counters of every
    kernel of the cycle (launches per cycle from the profile), against the
    compulsory state traffic 2 S(m) per cell-update (80 + 56 m bytes of
    persistent VNR state, read and written once)."""
    prof_file = ROOT / "profiles" / "kernel_counters_bisod_vnr.json"
    if not prof_file.exists():
        return None
    pj = json.loads(prof_file.read_text())
    table = pj.get(regime, {})
    table = table.get("kernels", table)
    cells = spec.nx * spec.ny
    nodes = (spec.nx + 1) * (spec.ny + 1)
    cycles = max(v[1] for k, v in kinds.items() if k in ("k_lag_cells", "k_final"))
    per_cell = 0.0
    for k, (ms, cnt) in kinds.items():
        kp = table.get(k) or table.get(k + "_pb") or table.get(k + "_f")
        if not kp:
            continue
        units = nodes if k in ("k_lag_nodes", "k_dual_grad", "k_dual_update") else cells
        per_cell += kp["dram_bytes_per_unit"] * units * (cnt / cycles) / cells
    compulsory = 2 * (80 + 56 * spec.nbmat)
    peaks = load_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    gbs = compulsory * cells / (ms_per_cycle * 1e-3) / 1e9
    return {"dram_bytes_per_cell": round(per_cell, 1), "compulsory_bytes_per_cell": compulsory,
            "over_compulsory": round(per_cell / compulsory, 2),
            "compulsory_gbs": gbs, "path_hbm_frac": gbs / hbm,
            "counters": f"profiles/kernel_counters_bisod_vnr.json [{regime}]"}


def port_developed(M, spec_fn, budget_s: float = 12.0) -> dict:
    """The C restatement in a developed flow: the same deck on 256^2,
    advanced until the waves cross most of the mesh, then timed per cycle
    (its work per cell grows once the cells leave the at-rest extrema)."""
    from oracle import port
    spec = spec_fn(256, 2400)
    run = port.PortRun(spec)
    run.step(1800)
    u = run.fetch("node_velocity").reshape(-1, 2)
    moving = float(np.mean((u[:, 0] != 0) | (u[:, 1] != 0)))
    n, t0 = 0, time.perf_counter()
    while n < 40 and time.perf_counter() - t0 < budget_s:
        run.step(1)
        n += 1
    el = time.perf_counter() - t0
    run.close()
    cores = port.num_threads()
    return {"value": spec.nx * spec.ny * n / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} cycles (1801..{1800 + n}) of the same deck on 256x256, "
                      f"{100 * moving:.0f}% of the nodes moving, {cores} OpenMP threads, "
                      f"{el:.1f} s"}


def bench_developed(M, ctx, args, local: int, K: int) -> dict:
    """The benchmark deck advanced untimed until most nodes move, then K
    cycles timed (CUDA events, state resident) and 4 profiled."""
    n = args.mesh
    adv = args.dev_advance
    spec = workload_spec(M, n, adv + K + 8)
    run = M.Run(spec, ctx)
    t0 = time.perf_counter()
    run.step(adv)
    adv_s = time.perf_counter() - t0
    u = run.fetch("node_velocity").reshape(-1, 2)
    moving = float(np.mean((u[:, 0] != 0) | (u[:, 1] != 0)))
    l0 = run.kernel_launches
    with Clocks(local) as clk:
        ms = run.timed(K)
    launches = run.kernel_launches - l0
    prof = run.profile(4)
    err = run.error()[0]
    run.close()
    kinds = {k: v for k, v in prof.items() if v[1] > 0}
    cells = n * n
    out = {"value": cells * K / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / K,
           "steps": K, "timed_cycles": [adv + 1, adv + K],
           "nodes_moving": moving, "advance_s": adv_s, "gpu_launches": launches,
           "error_word": err, "clocks": clk.summary(),
           "roofline": roofline_of(M, kinds, spec, "developed", local),
           "path": path_traffic(kinds, spec, "developed", ms / K),
           "kernel_ms": {k: [round(v[0], 4), v[1]] for k, v in kinds.items()}}
    if not args.no_cpu:
        out["cpu_baseline"] = port_developed(M, lambda m, c: workload_spec(M, m, c))
        out["vs_cpu"] = out["value"] / out["cpu_baseline"]["value"]
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
    cells = n * n
    # the K timed cycles end the configured window; the cycles before them
    # (at least W) run untimed and warm the graph, caches and clocks; 8 more
    # cycles after the window are profiled kernel by kernel
    adv, length = timed_window(K, W)
    run = M.Run(workload_spec(M, n, length + 8), ctx)
    run.step(adv)
    state_bytes = run.device_bytes
    launches0 = run.kernel_launches
    barrier_max(0.0, world)
    with Clocks(local) as clk:
        ms = run.timed(K)
    clocks = clk.summary()
    launches = run.kernel_launches - launches0
    ms = barrier_max(ms, world)
    value = cells * K * world / (ms * 1e-3)
    prof = run.profile(8)
    run.close()
    kinds = {k: v for k, v in prof.items() if v[1] > 0}
    spec = workload_spec(M, n, CYCLES)
    roofline = roofline_of(M, kinds, spec, "kernels", local)
    path = path_traffic(kinds, spec, "kernels", ms / K)
    # end to end through the C ABI with host buffers: the whole configured
    # job (creation with the device-built initial state, 200 cycles, fetch)
    t0 = time.perf_counter()
    e = M.Run(workload_spec(M, n, CYCLES), ctx)
    e.step(CYCLES)
    outs = [e.fetch(f) for f in ("density", "pressure", "energy", "fracvol_env",
                                 "node_velocity")]
    e2e_s = time.perf_counter() - t0
    h2d = CTRL_BYTES  # the control block; the initial state is built on the device
    d2h = sum(o.nbytes for o in outs)
    e.close()
    e2e = {"value": cells * CYCLES / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": h2d / CYCLES, "d2h_bytes_per_step": d2h / CYCLES,
           "includes": f"run creation (device-built initial state), all {CYCLES} "
                       "cycles, fetch of 5 fields"}
    if rank != 0:
        return
    cpu = None if args.no_cpu else cpu_baseline(lambda: workload_spec(M, n, CYCLES))
    developed = None if args.no_dev else bench_developed(M, ctx, args, local, K)
    batched = None if args.no_batch else bench_batch(M, ctx, args, local)
    eucclhyd = None if args.no_euc else bench_euc(M, ctx, args, local)
    served = None if args.no_serve else bench_serve(M, args, local)
    summary = {
        "plain": {"value": value, "e2e": e2e["value"], "window": [adv + 1, adv + K],
                  "dominant": roofline["kernel"], "hbm_frac": round(roofline["frac"], 3),
                  "path_hbm_frac": path and round(path["path_hbm_frac"], 3),
                  "vs_cpu": cpu and value / cpu["value"]},
    }
    if developed:
        summary["developed"] = {"value": developed["value"],
                                "nodes_moving": round(developed["nodes_moving"], 3),
                                "dominant": developed["roofline"]["kernel"],
                                "hbm_frac": round(developed["roofline"]["frac"], 3),
                                "vs_cpu": developed.get("vs_cpu")}
    if eucclhyd:
        summary["eucclhyd"] = {"value": eucclhyd["value"]}
    if served:
        summary["served"] = [[o["rate_req_s"], o["completed"], round((o["value"] or 0) / 1e6, 1),
                              round(o["p50_latency_s"] or 0, 3), round(o["p99_latency_s"] or 0, 3)]
                             for o in served["rates"]]
        summary["served_columns"] = ["rate_req_s", "completed", "M_cell_updates_s",
                                     "p50_s", "p99_s"]
    if batched:
        summary["batched"] = {"value": batched["value"],
                              "plain_mix": batched["plain_mix"]["value"],
                              "speedup_vs_plain_mix": batched["speedup_vs_plain_mix"],
                              "same_cycles": batched["timed_cycles"]}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": ms / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (analytic initial state)",
        "config": workload_config(K, W, n), "form": "plain",
        "window": [adv + 1, adv + K], "state_bytes": state_bytes,
        "e2e": e2e, "roofline": roofline, "path": path, "cpu_baseline": cpu,
        "clocks": clocks, "gpu_launches": launches,
        "kernel_ms": {k: [round(v[0], 4), v[1]] for k, v in kinds.items()},
        "served": served,
        "eucclhyd": eucclhyd,
        "developed": developed,
        "batched": batched,
        "summary": summary,
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
    ap.add_argument("--serve-rates", default="4,50,100,200,500,1000,2000")
    ap.add_argument("--serve-n", type=int, default=200)
    ap.add_argument("--serve-timeout", type=float, default=240.0)
    ap.add_argument("--dev-advance", type=int, default=4500)
    ap.add_argument("--no-dev", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
