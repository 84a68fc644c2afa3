"""Per-unit kernel counters from an ncu metrics capture (CSV log).

Turns the launch-by-metric rows that `ncu --metrics ... --csv --log-file`
writes for one captured cycle into the per-kernel, per-unit figures that
bench.py's roofline reads (DRAM bytes, FP64 flops and FP64-pipe instructions
per cell or node, the kernel's launch time under ncu):

python -m mahyco_gb300.ncu_counters --mesh 1024 \\
    --early counters_early.csv --developed counters_dev.csv \\
    --out profiles/kernel_counters_bisod_vnr.json

Units: cells (mesh^2), or nodes ((mesh+1)^2) for the node kernels; the
face-gradient kernel counts a face as a cell.  FP64 flops = dadd + dmul +
2 dfma thread instructions; FP64-pipe instructions = 32 x
sm__inst_executed_pipe_fp64 (arithmetic, division and square-root steps,
conversions and comparisons issued on that pipe).  ncu times are serialized
cold-cache launches: shares, not absolute speeds.
"""
from __future__ import annotations

import argparse
import csv
import json
import re
from collections import defaultdict

NODE_KERNELS = ("k_lag_nodes", "k_dual_grad", "k_dual_update")


def _value(s: str) -> float:
    return float(s.replace(",", ""))


def _name(kernel: str) -> str:
    m = re.search(r"(k_\w+)", kernel)
    return m.group(1) if m else kernel


def read_capture(path: str) -> dict[str, list[dict]]:
    """kernel name -> list of launches, each {metric: value}."""
    launches: dict[str, dict] = {}
    order: list[str] = []
    with open(path, newline="") as f:
        lines = [ln for ln in f if ln.startswith('"')]
    for row in csv.DictReader(lines):
        lid = row["ID"]
        if lid not in launches:
            launches[lid] = {"kernel": _name(row["Kernel Name"])}
            order.append(lid)
        unit = row.get("Metric Unit", "")
        val = _value(row["Metric Value"])
        metric = row["Metric Name"]
        # times to microseconds, bytes to bytes
        if metric == "gpu__time_duration.sum":
            val *= {"ns": 1e-3, "nsecond": 1e-3, "us": 1.0, "usecond": 1.0,
                    "ms": 1e3, "msecond": 1e3, "s": 1e6, "second": 1e6}.get(unit, 1.0)
        elif metric.startswith("dram__bytes"):
            scale = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "KB": 1e3,
                     "MB": 1e6, "GB": 1e9}.get(unit, 1)
            val *= scale
        launches[lid][metric] = val
    out: dict[str, list[dict]] = defaultdict(list)
    for lid in order:
        out[launches[lid]["kernel"]].append(launches[lid])
    return out


def summarize(capture: dict[str, list[dict]], mesh: int) -> dict:
    cells, nodes = mesh * mesh, (mesh + 1) * (mesh + 1)
    res = {}
    for k, ls in capture.items():
        n = len(ls)
        units = nodes if k in NODE_KERNELS else cells
        tot = lambda m: sum(l.get(m, 0.0) for l in ls)  # noqa: E731
        us = tot("gpu__time_duration.sum") / n
        dram = (tot("dram__bytes_read.sum") + tot("dram__bytes_write.sum")) / n
        flops = (tot("smsp__sass_thread_inst_executed_op_dadd_pred_on.sum")
                 + tot("smsp__sass_thread_inst_executed_op_dmul_pred_on.sum")
                 + 2 * tot("smsp__sass_thread_inst_executed_op_dfma_pred_on.sum")) / n
        res[k] = {
            "launches": n,
            "us_per_launch": round(us, 2),
            "dram_bytes_per_unit": round(dram / units, 2),
            "dram_gbs": round(dram / (us * 1e-6) / 1e9, 1) if us else None,
            "fp64_flops_per_unit": round(flops / units, 1),
            "dfma_per_unit": round(tot("smsp__sass_thread_inst_executed_op_dfma_pred_on.sum")
                                   / n / units, 1),
            "fp64_pipe_inst_per_unit": round(32 * tot("sm__inst_executed_pipe_fp64.sum")
                                             / n / units, 1),
            "fp64_tflops": round(flops / (us * 1e-6) / 1e12, 3) if us else None,
            "fp64_pipe_pct": round(tot("sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active")
                                   / n, 1),
            "warp_inst_per_unit": round(tot("sm__inst_executed.sum") / n / units, 2),
            "units": units,
        }
        # pipe and issue utilisation, when the capture has them
        for key, metric in (("alu_pipe_pct", "sm__pipe_alu_cycles_active.avg.pct_of_peak_sustained_active"),
                            ("fma_pipe_pct", "sm__pipe_fma_cycles_active.avg.pct_of_peak_sustained_active"),
                            ("issue_pct", "sm__inst_issued.avg.pct_of_peak_sustained_active")):
            if any(metric in l for l in ls):
                res[k][key] = round(tot(metric) / n, 1)
    return res


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--mesh", type=int, default=1024)
    ap.add_argument("--early", required=True)
    ap.add_argument("--developed", required=True)
    ap.add_argument("--out", required=True)
    ap.add_argument("--command", default="")
    ap.add_argument("--command-developed", default="")
    a = ap.parse_args()
    doc = {
        "workload": f"bi-material Sod Y, {a.mesh}x{a.mesh} cells, VNR order-2 remap, "
                    "superBee + PenteBorne pure, A1; the third cycle from the initial "
                    "state (the benchmark's regime), and one cycle of the developed flow "
                    "after 1200 cycles",
        "command": a.command,
        "command_developed": a.command_developed,
        "note": "per launch, divided by the launch's units (cells, or nodes for node "
                "kernels); FP64 flops = dadd + dmul + 2*dfma thread instructions; "
                "FP64-pipe inst = 32 x sm__inst_executed_pipe_fp64; alu / fma / issue: "
                "percent of peak sustained (active cycles); times are ncu's "
                "serialized cold-cache launches",
        "kernels": summarize(read_capture(a.early), a.mesh),
        "developed": summarize(read_capture(a.developed), a.mesh),
    }
    with open(a.out, "w") as f:
        json.dump(doc, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
