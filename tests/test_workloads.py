"""Seeded workload generators (CPU)."""
from __future__ import annotations

import collections

from mahyco_gb300.workloads import (MT19937_64, batch_mix, request_stream,
                                    state_bytes)


def test_mt19937_64_known_answer():
    g = MT19937_64()
    for _ in range(9999):
        g()
    assert g() == 9981545732273789042
    g = MT19937_64()
    assert [g() for _ in range(3)] == [14514284786278117030, 4620546740167642908,
                                       13109570281517897720]


def test_batch_mix_shape():
    mix = batch_mix()
    assert len(mix) == 512
    kinds = collections.Counter(i.kind for i in mix)
    assert kinds == {"sod": 171, "sedov": 171, "advection": 170}
    assert all(64 <= i.nx <= 1024 and 64 <= i.ny <= 256 for i in mix)
    assert all(i.cycles == 100 for i in mix)
    assert {i.limiter for i in mix} == {"minmod", "superBee"}
    # deterministic
    assert batch_mix()[:5] == mix[:5]
    assert sum(i.cells for i in mix) == sum(i.cells for i in batch_mix())


def test_request_stream():
    rs = request_stream(100.0, 300)
    gaps = [b.arrival - a.arrival for a, b in zip(rs, rs[1:])]
    assert all(g > 0 for g in gaps)
    mean = sum(gaps) / len(gaps)
    assert 0.007 < mean < 0.013  # Poisson at 100 req/s
    assert all(32 <= r.inst.nx <= 2048 and 32 <= r.inst.ny <= 2048 for r in rs)
    assert all(50 <= r.inst.cycles <= 500 for r in rs)
    assert {r.inst.nbmat for r in rs} == {1, 2, 3}
    assert all(r.inst.nbmat >= 2 for r in rs if r.inst.kind == "advection")
    assert state_bytes(rs[0].inst) == (80 + 56 * rs[0].inst.nbmat) * rs[0].inst.cells
