"""bench.py's roofline accounting on the CPU: the algorithmic bytes of the
dominant kernels (in general and for a cell at rest), the roofline fraction
from a launch time, and the cycle's DRAM bytes per cell from the committed
ncu counters."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


class _Spec:
    nx = ny = 2048
    nbmat = 2
    pb = 1


class _M:
    @staticmethod
    def fp64_peak_tflops(device):
        return 1.25


def test_algorithmic_bytes_of_the_lagrange_cell_kernel():
    # nb = 2, nc = 7: 21 state words in, 24 out
    assert bench.algorithmic_bytes("k_lag_cells", 2, True, rest=False) == 45 * 8
    # at rest: 4 unchanged stores, 4 rest-geometry loads and 5 geometry
    # stores left out, one flag byte read
    assert bench.algorithmic_bytes("k_lag_cells", 2, True, rest=True) == int((45 - 12.875) * 8)


def test_rest_accounting_only_lowers_the_kernels_that_skip_work():
    for k in ("k_final", "k_dual_update", "k_dual_grad", "k_lag_nodes"):
        assert (bench.algorithmic_bytes(k, 2, True, rest=True) ==
                bench.algorithmic_bytes(k, 2, True, rest=False)), k
    for k in ("k_lag_cells", "k_sweep_grad", "k_sweep_update"):
        assert (bench.algorithmic_bytes(k, 2, True, rest=True) <
                bench.algorithmic_bytes(k, 2, True, rest=False)), k
    # without PenteBorne the slope and update kernels keep their planes
    assert (bench.algorithmic_bytes("k_sweep_grad", 2, False, rest=True) ==
            bench.algorithmic_bytes("k_sweep_grad", 2, False, rest=False))


def test_roofline_fraction_from_a_launch_time():
    spec = _Spec()
    cells = spec.nx * spec.ny
    # two cycles' profile: the cell kernel dominates at 0.3 ms a launch
    kinds = {"k_lag_cells": (0.6, 2), "k_final": (0.36, 2), "k_lag_nodes": (0.24, 2)}
    r = bench.roofline_of(_M, kinds, spec, "kernels", 0)
    alg = bench.algorithmic_bytes("k_lag_cells", 2, True, rest=True) * cells
    assert r["kernel"] == "k_lag_cells"
    assert r["algorithmic_bytes_per_launch"] == alg
    assert r["achieved"] == pytest.approx(alg / 0.3e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    counters = json.loads((ROOT / "profiles" / "kernel_counters_bisod_vnr.json").read_text())
    per_unit = counters["kernels"]["k_lag_cells"]["dram_bytes_per_unit"]
    assert r["traffic"] == pytest.approx(per_unit * cells)
    # the counters' DRAM bytes are the algorithmic bytes within 10 %: nothing
    # is re-read
    assert abs(per_unit * cells / alg - 1.0) < 0.10


def test_cycle_dram_bytes_per_cell_from_the_counters():
    spec = _Spec()
    counters = json.loads((ROOT / "profiles" / "kernel_counters_bisod_vnr.json").read_text())
    table = counters["kernels"]
    # one cycle of the benchmark configuration: the launches per kind
    kinds = {k: (1.0, v["launches"]) for k, v in table.items()}
    p = bench.path_traffic(kinds, spec, "kernels", 1.0)
    cells = 1024 * 1024
    nodes = 1025 * 1025
    want = 0.0
    for k, v in table.items():
        units = nodes if k in ("k_lag_nodes", "k_dual_grad", "k_dual_update") else cells
        want += v["dram_bytes_per_unit"] * units * v["launches"] / cells
    # per-unit bytes of the 1024^2 capture applied to the 2048^2 units
    assert p["dram_bytes_per_cell"] == pytest.approx(want, rel=2e-3)
    assert p["compulsory_bytes_per_cell"] == 2 * (80 + 56 * 2)
    assert p["dram_bytes_per_cell"] < 2.0 * p["compulsory_bytes_per_cell"]


def test_timed_window_ends_the_configured_cycles():
    assert bench.timed_window(20, 5) == (180, 200)
    assert bench.timed_window(200, 5) == (5, 205)
