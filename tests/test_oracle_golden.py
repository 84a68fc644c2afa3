"""The C restatement (oracle/port) against golden vectors produced by the
reference itself (tests/golden/make_golden.py): bit-for-bit on every field."""
from __future__ import annotations

import pytest

from conftest import (CELL_FIELDS, GOLDEN, NODE_FIELDS, assert_bitwise,
                      fields_of, get_field, golden_cases, load_golden)


@pytest.mark.parametrize("case", golden_cases())
def test_port_matches_reference(case, port_lib):
    spec, meta, want = load_golden(GOLDEN / f"{case}.npz")
    run = port_lib.PortRun(spec)
    run.simulate()
    t, dt, n = run.time()
    assert n == int(meta["cycles"])
    assert t == float(meta["t"])
    for f in fields_of(spec):
        assert_bitwise(f"{case}:{f}", get_field(run, f, spec.nbmat), want[f])
