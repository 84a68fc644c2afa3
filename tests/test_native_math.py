"""Host-compiled checks of the kernels' scalar helpers (CPU, no GPU): the
integer-pipe comparisons and the one-division limiter must equal the IEEE
expressions of the reference bit for bit."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    pytest.skip("nvcc not available")


def test_integer_pipe_compares_and_limiter(tmp_path):
    exe = tmp_path / "check_int_compares"
    subprocess.run([_nvcc(), "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off",
                    "-I", str(ROOT / "include"), "-I", str(ROOT / "mahyco_gb300" / "csrc"),
                    "-x", "cu", str(ROOT / "tests" / "native" / "check_int_compares.cu"),
                    "-o", str(exe)], check=True, capture_output=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    assert " 0 mismatches; limiter" in res.stdout and " 0 mismatches; order3" in res.stdout
    assert res.stdout.rstrip().endswith(" 0 mismatches")


def test_integer_pipe_binary64_operations(tmp_path):
    """Products, sums, quotients and square roots formed on the integer
    pipe (the kernels' fast path for normal operands) equal the IEEE
    operations bit for bit: 12 M seeded cases plus edge values."""
    exe = tmp_path / "check_softfp"
    subprocess.run([_nvcc(), "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off",
                    "-I", str(ROOT / "include"), "-I", str(ROOT / "mahyco_gb300" / "csrc"),
                    "-x", "cu", str(ROOT / "tests" / "native" / "check_softfp.cu"),
                    "-o", str(exe)], check=True, capture_output=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    for op in ("mul", "add", "div", "sqrt", "div_by"):
        line = next(ln for ln in res.stdout.splitlines() if ln.startswith(op + ":"))
        assert line.endswith(" 0 mismatches"), line
        assert int(line.split()[1]) > 1_000_000, line  # the fast path is exercised
    assert res.stdout.rstrip().endswith("softfp: 0 mismatches")
