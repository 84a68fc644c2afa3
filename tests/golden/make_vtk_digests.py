"""Records the reference's own VTK output fixtures as digests.

For every deck of the reference's test suite that the GPU path takes (the
remap on, VNR or Eucclhyd), stores in tests/golden/vtk_digests.json:

  deck   the deck text as mahyco_gb300.deck_text writes it from the parsed
         options (checked to parse back to the same options)
  files  {file name: [size, sha256]} of every file in the case's
         reference/ directory (<module>.<call>.vtp, <module>.pvd), which the
         reference's test script compares with `diff -r output reference/`

The drop-in driver's test runs each deck and compares its output directory
with these digests, file by file.  Needs the reference sources; run from the
repo root:
  python tests/golden/make_vtk_digests.py --ref <reference tree>
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import mahyco_gb300 as M  # noqa: E402

OUT = Path(__file__).resolve().parent / "vtk_digests.json"


def digest(path: Path):
    data = path.read_bytes()
    return [len(data), hashlib.sha256(data).hexdigest()]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MAHYCO_REFERENCE"),
                    help="reference source tree (or set MAHYCO_REFERENCE)")
    a = ap.parse_args()
    if not a.ref:
        ap.error("the reference source tree is needed: --ref or MAHYCO_REFERENCE")
    cases = {}
    with tempfile.TemporaryDirectory() as tmp:
        for d in sorted((Path(a.ref) / "tests").iterdir()):
            deck = d / "donnees.txt"
            if not deck.exists() or not (d / "reference").is_dir():
                continue
            spec = M.parse_deck(deck)
            # every deck the GPU path takes: both schemes with the remap, VNR
            # without it (the Eucclhyd Lagrange-only deck is refused)
            if spec.scheme not in (M.SCHEME_VNR, M.SCHEME_EUCCLHYD):
                continue
            if spec.projection != 1 and spec.scheme != M.SCHEME_VNR:
                continue
            text = M.deck_text(spec)
            again = Path(tmp) / f"{d.name}.txt"
            again.write_text(text)
            assert M.parse_deck(again).as_dict() == spec.as_dict(), d.name
            files = {f.name: digest(f) for f in sorted((d / "reference").iterdir())}
            cases[d.name] = {"deck": text, "files": files}
    OUT.write_text(json.dumps(cases, indent=1, sort_keys=True) + "\n")
    print(f"{len(cases)} cases, {sum(len(c['files']) for c in cases.values())} files -> {OUT}")


if __name__ == "__main__":
    main()
