"""Generates the golden vectors under tests/golden/ from the REFERENCE itself.

Runs oracle/_ref/mahyco_dump (the unmodified MaHyCo sources compiled against
oracle/kokkos_shim by oracle/Makefile.ref) on input decks and stores the full
precision final state next to the option set parsed from the deck:

  tests/golden/<case>.npz   fields: density pressure energy sound_speed
                            pseudo divu cell_mass node_velocity node_mass
                            + *_env (nbmat columns), spec (JSON), meta

Cases: every deck of the reference's test suite that uses the remap
(AvecProjection = oui), VNR and Eucclhyd, plus decks derived from them: the
200x10 Sod workload, a reduced bi-material Sod with the mixed interface row,
and the three-material triple point with one exponent per material.
Eucclhyd fixtures hold cell_velocity instead of the VNR-only fields.

Needs the reference sources, given by --ref or MAHYCO_REFERENCE; run from
the repo root:
  make -f oracle/Makefile.ref REF=<reference tree> -j8
  python tests/golden/make_golden.py --ref <reference tree>
"""
from __future__ import annotations

import argparse
import json
import os
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
# what the harness dumps of a Eucclhyd run's initial state (--init-only: the
# pressure and sound speed are first formed by the first cycle)
FIELDS_EUC_INIT = ["density", "energy", "cell_velocity", "density_env", "energy_env",
                   "fracvol_env", "mass_fraction_env", "node_velocity"]
# what the harness dumps for a Eucclhyd run (the cell-centred velocity, the
# pressure and sound speed of the last cycle's start)
FIELDS_EUC = ["density", "pressure", "energy", "sound_speed", "cell_velocity",
              "density_env", "energy_env", "fracvol_env", "mass_fraction_env",
              "node_velocity"]

write_deck = M.write_deck


def run_reference(deck: Path, cycles: int = 0, extra=(), fields=FIELDS) -> dict:
    with tempfile.TemporaryDirectory() as d:
        args = [str(DUMP), str(deck), d]
        if cycles:
            args += ["--cycles", str(cycles)]
        args += list(extra)
        subprocess.run(args, stdout=subprocess.DEVNULL, check=True)
        meta = dict(line.split() for line in open(f"{d}/meta.txt"))
        out = {f: np.fromfile(f"{d}/{f}.f64") for f in fields}
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
    ap.add_argument("--ref", default=os.environ.get("MAHYCO_REFERENCE"),
                    help="reference source tree (or set MAHYCO_REFERENCE)")
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    if not a.ref:
        ap.error("the reference source tree is needed: --ref or MAHYCO_REFERENCE")
    tests = Path(a.ref) / "tests"
    if not DUMP.exists():
        sys.exit("oracle/_ref/mahyco_dump missing: make -f oracle/Makefile.ref")
    cases = []
    for d in sorted(tests.iterdir()):
        deck = d / "donnees.txt"
        if not deck.exists():
            continue
        spec = M.parse_deck(deck)
        # with the remap, and VNR without it (the Lagrange phase alone)
        if spec.projection == 1 or spec.scheme == M.SCHEME_VNR:
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
    # three-material triple point (Eucclhyd, superBee + PenteBorne mixte) with
    # one adiabatic exponent per material
    s = M.parse_deck(tests / "POINT_TRIPLE_SuperBee_PenteBorne_mixte" / "donnees.txt")
    s.gamma[0], s.gamma[1], s.gamma[2] = 1.5, 1.4, 1.5
    cases.append(("POINT_TRIPLE_gamma_1.5_1.4_1.5_pb_mixte", s,
                  tests / "POINT_TRIPLE_SuperBee_PenteBorne_mixte" / "donnees.txt",
                  ("--gamma", "1.5,1.4,1.5")))
    # order-3 projection with PenteBorne (mixte): the reference takes the
    # order-3 face value as an integrated flux and its state turns negative,
    # then NaN in the second cycle (it exits); one cycle pins that arithmetic
    src = (tests / "POINT_TRIPLE_SuperBee_PenteBorne_mixte" / "donnees.txt").read_text()
    lines = src.splitlines()
    for k, line in enumerate(lines):
        if line.startswith("# Ordre de la projection"):
            lines[k + 1] = "3"
    (tmp / "tp_o3_pb.txt").write_text("\n".join(lines) + "\n")
    s = M.parse_deck(tmp / "tp_o3_pb.txt")
    s.max_cycles = 1
    cases.append(("POINT_TRIPLE_o3_pb_mixte_1cycle", s, tmp / "tp_o3_pb.txt",
                  ("--cycles", "1")))
    # conservative projection (projectionConservative = oui, Eucclhyd): the
    # kinetic energy is remapped and corrects the internal energy
    # (eucclhyd_remap/PhaseRemapFinal.cc:115); no deck of the reference's
    # suite switches it on
    for src_case, name in (("SOD_X_bi_mat_Superbee_PenteBorne_pure", "SOD_X_bi_mat_Superbee_PB_pure_conservative"),
                           ("SOD_Y_bi_mat_MinMod_simple", "SOD_Y_bi_mat_MinMod_conservative"),
                           ("POINT_TRIPLE_SuperBee_PenteBorne_mixte", "POINT_TRIPLE_SuperBee_PB_mixte_conservative")):
        s = M.parse_deck(tests / src_case / "donnees.txt")
        s.projection_conservative = 1
        write_deck(s, tmp / f"{name}.txt")
        cases.append((name, s, tmp / f"{name}.txt", ()))
    # shock on a helium bubble (BiShockBubble, Eucclhyd): the gas enters
    # through the right side at the imposed velocity and the remap takes that
    # side's boundary flux (remap/BoundaryFluxes.cc), the one reference case
    # that switches computeBoundaryFluxes on; a 130x16 mesh of the
    # reference's 0.00125 deck at 0.005, exponents 1.4 / 1.667
    base = M.parse_deck(tests / "POINT_TRIPLE_MinMod_simple" / "donnees.txt")
    for lim, pb, order, cyc, tag in (("minmod", 0, 2, 120, "MinMod_o2"),
                                     ("superBee", 1, 2, 120, "SuperBee_PenteBorne_pure"),
                                     ("superBee", 0, 3, 60, "SuperBee_o3")):
        s = base.copy()
        s.test_case, s.nbmat = 14, 2
        s.nx, s.ny, s.dx, s.dy = 130, 16, 0.005, 0.005
        s.final_time, s.output_time = 1.0, 1.0
        s.gamma[0], s.gamma[1] = 1.4, 1.667
        s.limiter, s.pb, s.pb_mixte, s.pb_complet = M.LIMITERS[lim], pb, 0, 0
        s.projection_order = order
        s.max_cycles = cyc
        name = f"SHOCK_BUBBLE_{tag}"
        write_deck(s, tmp / f"{name}.txt")
        cases.append((name, s, tmp / f"{name}.txt",
                      ("--cycles", str(cyc), "--gamma", "1.4,1.667,1.4")))
    # Cases whose first cycle stops the reference: Noh and bi-material Noh
    # (no density initialisation: NaN in the remap final, "cell--Nan 0"),
    # the Eucclhyd unit tests (deltat_n stays 0: "pas de temps minimum") and
    # the VNR unit tests (e = 25 > 5: the energy abort).  Their initial state
    # is pinned (--init-only) and the stop is recorded beside it.
    init_cases = []
    base_e = M.parse_deck(tests / "SOD_X_Mono_mat_MinMod_simple" / "donnees.txt")
    base_v = M.parse_deck(tests / "SOD_X_Mono_mat_Minmod_vnr_o2" / "donnees.txt")
    # (stop, cell): what the reference prints when it stops in the first
    # cycle ("cell--Nan 0", "Fin de la simulation par pas de temps minimum",
    # "16 energie 25 ...")
    for name, base, tc, nb, nx, ny, stop in (
            ("NOH_euc_init", base_e, 6, 1, 40, 40, ("nan", 0)),
            ("BINOH_euc_init", base_e, 17, 2, 40, 40, ("nan", 0)),
            ("UNIT_euc_init", base_e, 0, 1, 40, 10, ("dt", -1)),
            ("BIUNIT_euc_init", base_e, 11, 2, 40, 10, ("dt", -1)),
            ("UNIT_vnr_init", base_v, 0, 1, 40, 10, ("energy", 16)),
            ("BIUNIT_vnr_init", base_v, 11, 2, 40, 10, ("energy", 16))):
        s = base.copy()
        s.test_case, s.nbmat, s.nx, s.ny = tc, nb, nx, ny
        s.dx, s.dy = 1.0 / nx, (1.0 / ny if ny == nx else 0.1)
        s.max_cycles = 0
        write_deck(s, tmp / f"{name}.txt")
        init_cases.append((name, s, tmp / f"{name}.txt", stop))
    for name, spec, deck, stop in init_cases:
        if a.only and a.only not in name:
            continue
        euc = spec.scheme == M.SCHEME_EUCCLHYD
        meta, fields = run_reference(deck, 0, ("--init-only",),
                                     FIELDS_EUC_INIT if euc else FIELDS)
        meta["init_only"] = "1"
        meta["reference_stop"], meta["reference_stop_cell"] = stop[0], str(stop[1])
        save(name, spec, meta, fields)
    for name, spec, deck, extra in cases:
        if a.only and a.only not in name:
            continue
        euc = spec.scheme == M.SCHEME_EUCCLHYD
        meta, fields = run_reference(deck, 0, extra, FIELDS_EUC if euc else FIELDS)
        save(name, spec, meta, fields)


if __name__ == "__main__":
    main()
