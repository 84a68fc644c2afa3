"""Generates the golden vectors under tests/golden/ from the REFERENCE itself.

Runs oracle/_ref/mahyco_dump (the unmodified MaHyCo sources compiled against
oracle/kokkos_shim by oracle/Makefile.ref) on input decks and stores the full
precision final state next to the option set parsed from the deck:

  tests/golden/<case>.npz   fields: density pressure energy sound_speed
                            pseudo divu cell_mass node_velocity node_mass
                            + *_env (nbmat columns), spec (JSON), meta

Cases: every VNR deck of the reference's test suite that uses the remap
(AvecProjection = oui), plus decks derived from them for the 200x10 Sod
workload and a reduced bi-material Sod with the mixed interface row.

Needs the reference sources (default /root/reference); run from the repo root:
  make -f oracle/Makefile.ref REF=/root/reference -j8
  python tests/golden/make_golden.py [--ref /root/reference]
"""
from __future__ import annotations

import argparse
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import mahyco_gb300 as M  # noqa: E402

OUT = Path(__file__).resolve().parent
DUMP = ROOT / "oracle" / "_ref" / "mahyco_dump"
FIELDS = ["density", "pressure", "energy", "sound_speed", "pseudo", "divu",
          "cell_mass", "density_env", "energy_env", "pressure_env",
          "fracvol_env", "mass_fraction_env", "node_velocity", "node_mass"]

LIM_NAME = {v: k for k, v in M.LIMITERS.items()}


def write_deck(spec: M.HydroSpec, path: Path) -> None:
    """Writes a positional deck (lecture_donnees/LectureDonnees.cc order)."""
    case_names = {0: "UnitTestCase", 1: "SedovTestCase", 2: "TriplePoint",
                  4: "SodCaseX", 5: "SodCaseY", 6: "NohTestCase",
                  7: "AdvectionX", 8: "AdvectionY", 9: "AdvectionVitX",
                  10: "AdvectionVitY", 11: "BiUnitTestCase",
                  12: "BiSedovTestCase", 13: "BiTriplePoint",
                  14: "BiShockBubble", 15: "BiSodCaseX", 16: "BiSodCaseY",
                  17: "BiNohTestCase", 18: "BiAdvectionX", 19: "BiAdvectionY",
                  20: "BiAdvectionVitX", 21: "BiAdvectionVitY"}
    on = lambda b: "oui" if b else "non"  # noqa: E731
    lines = ["# Cas test", case_names[spec.test_case],
             "# Nombre de Mailles en X", str(spec.nx),
             "# Nombre de Mailles en Y", str(spec.ny),
             "# DELTA_X", repr(spec.dx), "# DELTA_Y", repr(spec.dy),
             "# temps final", repr(spec.final_time),
             "# Temps entre deux sorties", repr(spec.output_time),
             "# Pas de temps initial", repr(spec.dt_init),
             "# Pas de temps minimal", repr(spec.dt_min)]
    for m in range(spec.nbmat):
        lines += ["# equation d'etat", "PerfectGas" if spec.eos[m] == 101 else "Void"]
    lines += ["# schema Lagrange", "VNR" if spec.scheme == 2001 else "Eucclhyd",
              "# ordre en espace", str(spec.space_order),
              "# avec projection", on(spec.projection),
              "# projection conservative", on(spec.projection_conservative),
              "# Limite fraction volumique", repr(spec.threshold),
              "# Ordre de la projection", str(spec.projection_order),
              "# Limiteurs", LIM_NAME[spec.limiter],
              "# option Pente Borne", on(spec.pb)]
    if spec.pb:
        lines += ["# Pente Borne mixte", on(spec.pb_mixte),
                  "# limiteur mailles pures", LIM_NAME.get(spec.limiter_pure, "minmod"),
                  "# Pente Borne complet", on(spec.pb_complet)]
    if spec.scheme == 2001:
        lines += ["# pseudo_centree", on(spec.pseudo_centree)]
        if spec.projection:
            lines += ["# methode flux masse", ["A1", "A2", "PB"][spec.dual_mass_flux]]
    path.write_text("\n".join(lines) + "\n")


def run_reference(deck: Path, cycles: int = 0, extra=()) -> dict:
    with tempfile.TemporaryDirectory() as d:
        args = [str(DUMP), str(deck), d]
        if cycles:
            args += ["--cycles", str(cycles)]
        args += list(extra)
        subprocess.run(args, stdout=subprocess.DEVNULL, check=True)
        meta = dict(line.split() for line in open(f"{d}/meta.txt"))
        out = {f: np.fromfile(f"{d}/{f}.f64") for f in FIELDS}
    return meta, out


def save(case: str, spec: M.HydroSpec, meta: dict, fields: dict) -> None:
    nb = spec.nbmat
    arrays = {}
    for f, a in fields.items():
        if f.endswith("_env"):
            a = a.reshape(-1, 3)[:, :nb].copy()
        arrays[f] = a
    np.savez_compressed(OUT / f"{case}.npz", spec=json.dumps(spec.as_dict()),
                        meta=json.dumps(meta), **arrays)
    print(f"{case}: {meta['cycles']} cycles, t={meta['t']}")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    tests = Path(a.ref) / "tests"
    if not DUMP.exists():
        sys.exit("oracle/_ref/mahyco_dump missing: make -f oracle/Makefile.ref")
    cases = []
    for d in sorted(tests.iterdir()):
        deck = d / "donnees.txt"
        if not deck.exists():
            continue
        spec = M.parse_deck(deck)
        if spec.scheme == M.SCHEME_VNR and spec.projection == 1:
            cases.append((d.name, spec, deck, ()))
    tmp = Path(tempfile.mkdtemp())
    # 200x10 Sod X, VNR, order-2 remap, minmod, t = 0.2
    s = M.parse_deck(tests / "SOD_X_Mono_mat_Minmod_vnr_o2" / "donnees.txt")
    s.ny, s.dy = 10, 0.01
    write_deck(s, tmp / "sod200x10.txt")
    cases.append(("SOD_X_200x10_vnr_o2_minmod", s, tmp / "sod200x10.txt", ()))
    # bi-material Sod Y, superBee + PenteBorne pure, 64x64, mixed interface row
    s = M.parse_deck(tests / "SOD_Y_bi_mat_Superbee_PenteBorne_pure_vnr" / "donnees.txt")
    s.nx, s.ny, s.dx, s.dy = 64, 64, 1.0 / 64, 1.0 / 64
    write_deck(s, tmp / "bisod64.txt")
    s.init_variant = 1
    cases.append(("BISOD_Y_64x64_superbee_pb_mixedrow", s, tmp / "bisod64.txt",
                  ("--ext-mixed-row",)))
    for name, spec, deck, extra in cases:
        if a.only and a.only not in name:
            continue
        meta, fields = run_reference(deck, 0, extra)
        save(name, spec, meta, fields)


if __name__ == "__main__":
    main()
