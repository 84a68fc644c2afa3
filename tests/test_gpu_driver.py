"""The drop-in driver (mahyco_gb300_run <deck>) against the reference's own
test suite: for every deck the GPU path takes (VNR and Eucclhyd with the
remap), the output directory must equal the reference's committed
reference/ directory file for file -- the check the reference's
tests/launch_test.sh makes with `diff -r output reference/`.  The reference
files are held as sizes + SHA-256 digests (tests/golden/vtk_digests.json,
made by tests/golden/make_vtk_digests.py)."""
from __future__ import annotations

import hashlib
import json
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = json.loads((GOLDEN / "vtk_digests.json").read_text())


@pytest.fixture(scope="module")
def driver():
    from mahyco_gb300 import build
    import mahyco_gb300 as M
    build.build()
    exe = Path(M.driver_path())
    assert exe.exists(), "driver not built"
    return exe


def digests(d: Path):
    return {f.name: [f.stat().st_size, hashlib.sha256(f.read_bytes()).hexdigest()]
            for f in sorted(d.iterdir())}


def _deck(tmp_path, case):
    p = tmp_path / f"{case}.txt"
    p.write_text(CASES[case]["deck"])
    return p


@pytest.mark.parametrize("case", sorted(CASES))
def test_driver_output_matches_reference_files(driver, case, tmp_path):
    deck = _deck(tmp_path, case)
    res = subprocess.run([str(driver), str(deck), "--quiet"], cwd=tmp_path,
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    got = digests(tmp_path / "output")
    want = {k: list(v) for k, v in CASES[case]["files"].items()}
    assert sorted(got) == sorted(want), (sorted(set(got) - set(want)),
                                         sorted(set(want) - set(got)))
    bad = [f for f in want if got[f] != want[f]]
    assert not bad, f"{len(bad)} of {len(want)} files differ: {bad[:5]}"


def test_driver_output_dir_and_none(driver, tmp_path):
    """--output-dir BASE writes BASE/output; "none" writes nothing
    (cppnabla/mesh/FileWriter.cc:20-35)."""
    case = "SOD_X_Mono_mat_Minmod_vnr_o2"
    deck = _deck(tmp_path, case)
    base = tmp_path / "b"
    base.mkdir()
    (base / "output").mkdir()
    (base / "output" / "stale.vtp").write_text("x")  # emptied first, as the reference does
    res = subprocess.run([str(driver), str(deck), "--output-dir", str(base), "--quiet"],
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    assert digests(base / "output") == {k: list(v) for k, v in CASES[case]["files"].items()}
    none = tmp_path / "n"
    none.mkdir()
    res = subprocess.run([str(driver), str(deck), "--output-dir", "none", "--quiet"],
                         cwd=none, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    assert not any(none.iterdir())


def test_driver_rejects_bad_deck_and_eucclhyd_lagrange_only(driver, tmp_path):
    """A deck that does not parse exits 1; an Eucclhyd run without the remap
    (the one reference deck the GPU path does not take) is refused at
    creation with exit 2."""
    import mahyco_gb300 as M
    bad = tmp_path / "bad.txt"
    bad.write_text("# Cas test\nNotACase\n")
    res = subprocess.run([str(driver), str(bad)], cwd=tmp_path, capture_output=True,
                         text=True, timeout=120)
    assert res.returncode == 1
    spec = M.parse_deck(_deck(tmp_path, "POINT_TRIPLE_MinMod_simple"))
    spec.projection = 0
    lag = tmp_path / "lag.txt"
    M.write_deck(spec, lag)
    res = subprocess.run([str(driver), str(lag)], cwd=tmp_path, capture_output=True,
                         text=True, timeout=120)
    assert res.returncode == 2 and "remap" in res.stderr


@pytest.mark.parametrize("case", ["SOD_Y_bi_mat_Superbee_PenteBorne_pure_vnr",
                                  "POINT_TRIPLE_MinMod_simple"])
def test_step_to_output_pauses_at_dump_times(case, tmp_path):
    """hydro_run_step_to_output stops exactly before the cycles whose start
    time meets the dump condition: the same cycles a cycle-by-cycle loop
    finds, with bit-identical states."""
    import mahyco_gb300 as M
    spec = M.parse_deck(_deck(tmp_path, case))
    a, b = M.Run(spec), M.Run(spec)
    seen_a, seen_b = [], []
    last = 0.0
    while True:  # cycle by cycle
        t, _, n = a.time()
        if t >= last + spec.output_time or t == 0.0:
            seen_a.append((n, t))
            last = t
        if a.step(1):
            break
    last = 0.0
    while True:  # paused by the device
        t, _, n = b.time()
        if t >= last + spec.output_time or t == 0.0:
            seen_b.append((n, t))
            last = t
        done, paused = b.step_to_output(1 << 20, last + spec.output_time)
        if done:
            break
        assert paused
    assert seen_a == seen_b and len(seen_a) > 3
    for f in ("density", "energy", "fracvol_env"):
        assert (a.fetch(f) == b.fetch(f)).all(), f
    assert a.time() == b.time()
