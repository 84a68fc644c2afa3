"""The fused remap sweep (opt-in: MAHYCO_GB300_FUSED_SWEEPS=1 at run
creation) against the reference and against the default kernels: every
PenteBorne VNR deck of the reference's suite through the drop-in driver
gives the reference's output directory byte for byte, and the benchmark's
options on a 256^2 mesh give the same state as the separate slope and
update kernels, bit for bit, on every field."""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import CELL_FIELDS, NODE_FIELDS, get_field

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = json.loads((GOLDEN / "vtk_digests.json").read_text())
PB_VNR = sorted(k for k in CASES if "PenteBorne" in k and "vnr" in k)


@pytest.fixture(scope="module")
def driver():
    from mahyco_gb300 import build
    import mahyco_gb300 as M
    build.build()
    return Path(M.driver_path())


@pytest.mark.parametrize("case", PB_VNR)
def test_fused_sweep_driver_output_matches_reference(driver, case, tmp_path):
    deck = tmp_path / f"{case}.txt"
    deck.write_text(CASES[case]["deck"])
    env = dict(os.environ, MAHYCO_GB300_FUSED_SWEEPS="1")
    res = subprocess.run([str(driver), str(deck), "--quiet"], cwd=tmp_path, env=env,
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    out = tmp_path / "output"
    got = {f.name: [f.stat().st_size, hashlib.sha256(f.read_bytes()).hexdigest()]
           for f in sorted(out.iterdir())}
    want = {k: list(v) for k, v in CASES[case]["files"].items()}
    bad = [f for f in want if got.get(f) != want[f]]
    assert sorted(got) == sorted(want) and not bad, bad[:5]


def test_fused_sweep_equals_separate_kernels():
    import mahyco_gb300 as M
    from mahyco_gb300 import build
    from bench import workload_spec
    build.build()
    spec = workload_spec(M, 256, 120)
    plain = M.Run(spec)
    os.environ["MAHYCO_GB300_FUSED_SWEEPS"] = "1"
    try:
        fused = M.Run(spec)
    finally:
        del os.environ["MAHYCO_GB300_FUSED_SWEEPS"]
    for run in (plain, fused):
        run.step(120)
    assert plain.time() == fused.time()
    for f in CELL_FIELDS + NODE_FIELDS:
        a, b = get_field(plain, f, spec.nbmat), get_field(fused, f, spec.nbmat)
        assert np.array_equal(np.ascontiguousarray(a).view(np.uint64),
                              np.ascontiguousarray(b).view(np.uint64)), f
