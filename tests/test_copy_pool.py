"""The host copy threads of the field fetch (CPU, no GPU): back-to-back
copies of random sizes and alignments with 0 to 7 workers land exactly in
their destination range."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_copy_pool(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = tmp_path / "check_copy_pool"
    subprocess.run([cxx, "-std=c++17", "-O2", "-pthread", "-Wall",
                    "-I", str(ROOT / "mahyco_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "check_copy_pool.cc"), "-o", str(exe)],
                   check=True, capture_output=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert res.stdout.strip() == "copy_pool: 960 jobs, 0 mismatches"
