"""Serving loop (hydro_serve_*): requests arriving over time are admitted
against the HBM budget, advanced together and retired at their own end; each
result must equal the same run advanced alone, bit for bit."""
from __future__ import annotations

import time

import pytest

from conftest import CELL_FIELDS, NODE_FIELDS, assert_bitwise, get_field

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    import mahyco_gb300
    from mahyco_gb300 import build
    build.build()
    return mahyco_gb300


def small_stream(n, rate, seed):
    from mahyco_gb300.workloads import request_stream
    return request_stream(rate, n, seed=seed, size_range=(12, 96), cycle_range=(5, 40))


def compare_alone(M, served, spec, tag):
    alone = M.Run(spec, M.Context(0))
    alone.simulate()
    for f in CELL_FIELDS + NODE_FIELDS + ["node_mass"]:
        assert_bitwise(f"{tag}:{f}", get_field(served, f, spec.nbmat),
                       get_field(alone, f, spec.nbmat))
    assert served.time() == alone.time(), tag


def drain(server, n, timeout=120.0, order=None):
    out, t0 = {}, time.time()
    while len(out) < n:
        d = server.poll(1.0)
        if d is not None:
            out[d.req_id] = (d.status, d.latency_s, d.cycles, d.cells)
            if order is not None:
                order.append(d.req_id)
        assert time.time() - t0 < timeout, "serving did not finish"
    return out


def test_served_equals_alone(M):
    ctx = M.Context(0)
    srv = M.Server(ctx, tick_cycles=4)
    reqs = small_stream(18, 400.0, seed=21)
    ids, specs = [], {}
    t0 = time.perf_counter()
    for r in reqs:  # Poisson arrivals while earlier runs are on the GPU
        dt = r.arrival - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        spec = r.inst.spec(M)
        rid = srv.submit(spec, keep=True)
        ids.append(rid)
        specs[rid] = (spec, r.inst)
    done = drain(srv, len(ids))
    st = srv.stats()
    assert st["completed"] == len(ids) and st["failed"] == 0
    assert st["peak_resident"] > 1  # work of different requests overlapped
    for rid in ids:
        status, lat, cycles, cells = done[rid]
        spec, inst = specs[rid]
        assert status & ~M.ERR_NEGATIVE == 0
        assert lat > 0.0 and cells == inst.nx * inst.ny
        assert cycles == inst.cycles
        compare_alone(M, srv.result(rid), spec, f"req{rid}")
        srv.release(rid)
    srv.stop()


def test_budget_admission(M):
    """With room for about two runs at a time, requests wait in arrival
    order; the bytes held never exceed the budget."""
    ctx = M.Context(0)
    from mahyco_gb300.workloads import Instance
    insts = [Instance("sod", 64, 48, 2, "minmod", 30, "X") for _ in range(6)]
    spec0 = insts[0].spec(M)
    one = M.Run(spec0, ctx)
    per_run = one.device_bytes
    one.close()
    budget = int(2.5 * per_run)
    srv = M.Server(ctx, budget=budget, tick_cycles=4)
    ids = [srv.submit(i.spec(M), keep=False) for i in insts]
    order = []
    drain(srv, len(ids), order=order)
    st = srv.stats()
    assert st["completed"] == 6
    assert st["peak_bytes"] <= budget
    assert st["peak_resident"] <= 2
    # first come, first served: completions come back in arrival order
    assert order == ids
    srv.stop()


def test_result_independent_of_mix(M):
    """The same request served with two different sets of companions gives
    identical results."""
    from mahyco_gb300.workloads import Instance
    probe = Instance("sedov", 40, 36, 1, "superBee", 25)
    results = []
    for seed in (1, 2):
        ctx = M.Context(0)
        srv = M.Server(ctx, tick_cycles=3)
        others = small_stream(6, 1000.0, seed=seed)
        for r in others[:3]:
            srv.submit(r.inst.spec(M))
        rid = srv.submit(probe.spec(M), keep=True)
        for r in others[3:]:
            srv.submit(r.inst.spec(M))
        drain(srv, 7)
        run = srv.result(rid)
        results.append({f: run.fetch(f) for f in ("density", "energy", "node_velocity")})
        srv.release(rid)
        srv.stop()
    for f in results[0]:
        assert_bitwise(f, results[0][f], results[1][f])


def test_invalid_request_fails_alone(M):
    ctx = M.Context(0)
    srv = M.Server(ctx)
    from mahyco_gb300.workloads import Instance
    good = Instance("sod", 32, 32, 1, "minmod", 10, "Y").spec(M)
    bad = good.copy()
    bad.nx = 1  # an invalid mesh: rejected at preparation, on the worker
    a = srv.submit(good)
    b = srv.submit(bad)
    done = drain(srv, 2)
    assert done[a][0] == 0
    assert done[b][0] == -1
    # a run without the remap is refused at submission (the serving loop
    # advances runs with the remap), and the loop goes on
    lag = good.copy()
    lag.projection = 0
    with pytest.raises(RuntimeError, match="remap"):
        srv.submit(lag)
    c = srv.submit(good)
    assert drain(srv, 1)[c][0] == 0
    srv.stop()


def test_served_eucclhyd_equals_alone(M):
    """Eucclhyd requests are served beside VNR ones (the batch's phase
    kernels of each scheme skip the other's tiles): each result equals the
    same run alone."""
    from conftest import GOLDEN, fields_of, golden_cases, init_only, load_golden
    ctx = M.Context(0)
    srv = M.Server(ctx, tick_cycles=4)
    euc = [c for c in golden_cases()
           if load_golden(GOLDEN / f"{c}.npz")[0].scheme == M.SCHEME_EUCCLHYD
           and load_golden(GOLDEN / f"{c}.npz")[0].projection == 1
           and not init_only(load_golden(GOLDEN / f"{c}.npz")[1])][:4]
    specs = [load_golden(GOLDEN / f"{c}.npz")[0] for c in euc]
    for r in small_stream(4, 1000.0, seed=5):
        specs.append(r.inst.spec(M))
    ids = [srv.submit(s, keep=True) for s in specs]
    done = drain(srv, len(ids), timeout=600.0)
    for rid, s in zip(ids, specs):
        assert done[rid][0] & ~M.ERR_NEGATIVE == 0
        served = srv.result(rid)
        alone = M.Run(s, M.Context(0))
        alone.simulate()
        for f in fields_of(s):
            assert_bitwise(f"req{rid}:{f}", get_field(served, f, s.nbmat),
                           get_field(alone, f, s.nbmat))
        assert served.time() == alone.time()
        srv.release(rid)
    srv.stop()
