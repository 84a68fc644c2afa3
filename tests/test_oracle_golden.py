"""The C restatement (oracle/port) against golden vectors produced by the
reference itself (tests/golden/make_golden.py): bit-for-bit on every field."""
from __future__ import annotations

import pytest

from conftest import (GOLDEN, assert_bitwise, check_first_cycle_stop, fields_of,
                      get_field, golden_cases, init_fields_of, init_only,
                      load_golden)


@pytest.mark.parametrize("case", golden_cases())
def test_port_matches_reference(case, port_lib):
    spec, meta, want = load_golden(GOLDEN / f"{case}.npz")
    run = port_lib.PortRun(spec)
    if init_only(meta):
        # the reference stops in the first cycle: its initial state, then
        # the same stop
        assert run.time() == (0.0, float(meta["dt"]), 0)
        for f in init_fields_of(spec):
            assert_bitwise(f"{case}:{f}", get_field(run, f, spec.nbmat), want[f])
        check_first_cycle_stop(run, meta)
        return
    run.simulate()
    t, dt, n = run.time()
    assert n == int(meta["cycles"])
    assert t == float(meta["t"])
    for f in fields_of(spec):
        assert_bitwise(f"{case}:{f}", get_field(run, f, spec.nbmat), want[f])
