"""The C-ABI library loads and exports every function include/hydro_gb300.h
declares (no GPU needed: nothing is called that touches the device)."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "hydro_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hydro_\w+)\s*\(", text)))


def test_library_exports_declared_symbols():
    from mahyco_gb300 import build
    lib_path = build.build()
    lib = ctypes.CDLL(str(lib_path))
    names = declared_functions()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_spec_defaults_and_deck_parse(tmp_path):
    import mahyco_gb300 as M
    s = M.default_spec()
    assert s.threshold == 1e-16 and s.projection_order == 2 and s.pseudo_centree == 1
    assert s.cfl == 0.45 and s.dt_min == 1e-10 and list(s.gamma) == [1.4] * 3
    deck = tmp_path / "d.txt"
    deck.write_text("# c\nBiSodCaseY\n# nx\n5\n# ny\n200\n# dx\n0.02\n# dy\n"
                    "0.005\n# tf\n0.2\n# out\n1.e-2\n# dt\n1.e-4\n# dtmin\n"
                    "1.e-12\n# eos\nPerfectGas\n# eos\nPerfectGas\n# schema\nVNR\n"
                    "# ordre\n2\n# proj\noui\n# cons\nnon\n# seuil\n1.e-16\n"
                    "# ordre proj\n2\n# lim\nsuperBee\n# pb\noui\n# mixte\nnon\n"
                    "# pure\narithmeticG\n# complet\nnon\n# pseudo\nnon\n")
    s = M.parse_deck(deck)
    assert (s.test_case, s.nbmat, s.nx, s.ny) == (16, 2, 5, 200)
    assert (s.limiter, s.pb, s.limiter_pure, s.pb_complet) == (301, 1, 1303, 0)
    # the dual mass-flux key is absent: the reference re-reads the previous
    # word ("non"), which maps to 0 = A1
    assert s.dual_mass_flux == 0 and s.pseudo_centree == 0
    assert s.dy == 0.005 and s.final_time == 0.2


def test_unknown_limiter_is_rejected(tmp_path):
    import mahyco_gb300 as M
    import pytest
    deck = tmp_path / "d.txt"
    deck.write_text("# c\nSodCaseX\n# nx\n5\n# ny\n5\n# dx\n0.1\n# dy\n0.1\n# tf\n"
                    "0.2\n# out\n1\n# dt\n1\n# dtmin\n1\n# eos\nPerfectGas\n"
                    "# schema\nVNR\n# o\n2\n# p\noui\n# c\nnon\n# s\n1e-16\n"
                    "# op\n2\n# lim\nnotalimiter\n")
    with pytest.raises(RuntimeError, match="limiter"):
        M.parse_deck(deck)
