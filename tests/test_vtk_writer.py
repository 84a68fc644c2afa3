"""The drop-in driver's VTK writer on the CPU (no GPU): its number
formatting equals std::ostream's default formatting (what the reference's
PvdFileWriter2D uses) on ~3M values including every special value, and its
output for a given set of fields is byte-identical to the reference's own
fixture files -- the first output of several reference decks, whose fields
(the initial state) come from the oracle."""
from __future__ import annotations

import hashlib
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
CASES = json.loads((GOLDEN / "vtk_digests.json").read_text())


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = tmp_path_factory.mktemp("h") / "vtk_writer_harness"
    tools = ROOT / "mahyco_gb300" / "tools_src"
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-ffp-contract=off",
                    "-I", str(tools), str(ROOT / "tests" / "native" / "vtk_writer_harness.cc"),
                    str(tools / "pvd_writer.cc"), "-o", str(exe)],
                   check=True, capture_output=True)
    return exe


def test_formatting_equals_ostream(harness):
    res = subprocess.run([str(harness), "selftest"], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert " 0 mismatches" in res.stdout


def _vnr_first_output(case, tmp_path):
    """Writes call 1 (t = 0) of a VNR deck from the oracle's initial state."""
    import mahyco_gb300 as M
    from oracle.port import PortRun
    deck = tmp_path / "deck.txt"
    deck.write_text(CASES[case]["deck"])
    s = M.parse_deck(deck)
    r = PortRun(s)
    fields = {"Pressure": r.fetch("pressure"), "Density": r.fetch("density"),
              "Energy": r.fetch("energy")}
    fv = r.fetch("fracvol_env").reshape(-1, 3)
    if s.nbmat > 1:
        fields["fracvol1"] = fv[:, 0].copy()
    if s.nbmat > 2:
        fields["fracvol2"] = fv[:, 1].copy()
    u = r.fetch("node_velocity").reshape(-1, 2)
    nodes = {"VitesseX": u[:, 0].copy(), "VitesseY": u[:, 1].copy()}
    parts = ["dump", "1", (0.0).hex(), str(len(fields))]
    for k, (name, a) in enumerate(list(fields.items()) + list(nodes.items())):
        p = tmp_path / f"f{k}.bin"
        np.ascontiguousarray(a).tofile(p)
        if k == len(fields):
            parts.append(str(len(nodes)))
        parts += [name, str(p)]
    return s, " ".join(parts) + "\n"


@pytest.mark.parametrize("case", ["SOD_X_Mono_mat_Minmod_vnr_o2",
                                  "SOD_Y_bi_mat_Superbee_PenteBorne_pure_vnr",
                                  "ADVECTION_VITX_bi_mat_Superbee_A1_vnr"])
def test_first_output_matches_reference_file(harness, case, tmp_path, port_lib):
    s, line = _vnr_first_output(case, tmp_path)
    subprocess.run([str(harness), "series", str(tmp_path), "VnrRemap", str(s.nx), str(s.ny),
                    s.dx.hex(), s.dy.hex()], input=line, text=True, check=True, timeout=120)
    data = (tmp_path / "output" / "VnrRemap.1.vtp").read_bytes()
    want = CASES[case]["files"]["VnrRemap.1.vtp"]
    assert [len(data), hashlib.sha256(data).hexdigest()] == want


def test_particle_file_layout(harness, tmp_path):
    """An Eucclhyd output writes the empty particle file beside the mesh file
    (eucclhyd_remap/EucclhydRemap.cc:55-58): no points, no polygons, the
    variable names only; both series list the call in their .pvd."""
    n = 6
    for k, name in enumerate(["Density", "Pressure"]):
        np.full(n, 0.5 * (k + 1)).tofile(tmp_path / f"{name}.bin")
    line = (f"dump 1 {(0.0).hex()} 2 Density {tmp_path}/Density.bin "
            f"Pressure {tmp_path}/Pressure.bin 0\n")
    subprocess.run([str(harness), "series", str(tmp_path), "EucclhydRemap", "3", "2",
                    (0.5).hex(), (0.25).hex(), "--particles"], input=line, text=True,
                   check=True, timeout=60)
    out = tmp_path / "output"
    assert sorted(p.name for p in out.iterdir()) == [
        "EucclhydRemap.1.vtp", "EucclhydRemap.pvd", "Particules.1.vtp", "Particules.pvd"]
    part = (out / "Particules.1.vtp").read_text().splitlines()
    assert part[3] == '\t\t<Piece NumberOfPoints="0" NumberOfPolys="0">'
    assert '\t\t\t<PointData Scalars="VolumePart">' in part
    assert '\t\t\t<CellData Scalars="Density">' in part
    mesh = (out / "EucclhydRemap.1.vtp").read_text().splitlines()
    assert mesh[6] == (" 0 0 0 0.5 0 0 1 0 0 1.5 0 0 0 0.25 0 0.5 0.25 0 1 0.25 0 1.5 0.25 0"
                       " 0 0.5 0 0.5 0.5 0 1 0.5 0 1.5 0.5 0")
    assert mesh[11] == "  0 1 5 4  1 2 6 5  2 3 7 6  4 5 9 8  5 6 10 9  6 7 11 10"
    assert mesh[14] == " 4 8 12 16 20 24"
    assert "PointData" not in "".join(mesh)
    pvd = (out / "EucclhydRemap.pvd").read_text()
    assert '<DataSet timestep="0" group="" part="0" file="EucclhydRemap.1.vtp"/>' in pvd
