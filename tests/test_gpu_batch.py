"""Batched execution (hydro_batch_step) against the plain path and the oracle.

The batch changes only which thread computes which item, so every run of a
batch must end bit-identical to the same run advanced alone, whatever the
tile widths and grids the autotuner picks, and to the C restatement.
"""
from __future__ import annotations

import pytest

from conftest import (CELL_FIELDS, GOLDEN, NODE_FIELDS, STOP_BITS, assert_bitwise,
                      fields_of, get_field, golden_cases, init_only, load_golden)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    import mahyco_gb300
    from mahyco_gb300 import build
    build.build()
    return mahyco_gb300


def small_mix(n, seed):
    from mahyco_gb300.workloads import batch_mix
    return batch_mix(n, seed=seed, cycles=40, nx_range=(16, 160), ny_range=(12, 72))


def compare_runs(M, a, b, nbmat, tag):
    for f in CELL_FIELDS + NODE_FIELDS + ["node_mass"]:
        assert_bitwise(f"{tag}:{f}", get_field(a, f, nbmat), get_field(b, f, nbmat))
    assert a.time() == b.time(), tag
    assert a.error() == b.error(), tag


def test_batch_matches_plain_mixed_kinds(M):
    """A seeded mix of Sod, Sedov and advection runs of uneven sizes, run for
    40 cycles in one batch (the first cycles tune the launches) and one by
    one through the plain path."""
    ctx = M.Context(0)
    mix = small_mix(24, seed=11)
    specs = [inst.spec(M) for inst in mix]
    batched = [M.Run(s, ctx) for s in specs]
    batch = M.Batch(batched)
    left = batch.step(40)
    assert left == 0  # every run stops at its 40-cycle cap
    cfg = batch.config()
    assert cfg["tuned"]
    for inst, s, rb in zip(mix, specs, batched):
        alone = M.Run(s, ctx)
        alone.simulate()
        compare_runs(M, rb, alone, s.nbmat, f"{inst.kind}{inst.nx}x{inst.ny}")
        assert rb.time()[2] == 40


def test_batch_matches_oracle(M, port_lib):
    from oracle.port import PortRun
    ctx = M.Context(0)
    mix = small_mix(6, seed=5)
    specs = [inst.spec(M) for inst in mix]
    runs = [M.Run(s, ctx) for s in specs]
    M.Batch(runs).step(40)
    for inst, s, r in zip(mix, specs, runs):
        ref = PortRun(s)
        ref.step(40)
        for f in ["density", "pressure", "energy", "pseudo", "fracvol_env",
                  "density_env", "node_velocity"]:
            want = ref.fetch(f)
            if f.endswith("_env"):
                want = want.reshape(-1, 3)[:, :s.nbmat]
            assert_bitwise(f"{inst.kind}:{f}", get_field(r, f, s.nbmat), want)
        assert r.time() == ref.time()


def test_batch_of_reference_decks(M):
    """Every VNR golden deck (orders 1-3, PenteBorne pure / complet, A1 / A2 /
    PB dual fluxes, one to two materials, advection and Sod) in one batch: runs
    end at their own final times and match the reference's final state."""
    ctx = M.Context(0)
    cases = [c for c in golden_cases()
             if load_golden(GOLDEN / f"{c}.npz")[0].scheme == M.SCHEME_VNR
             and load_golden(GOLDEN / f"{c}.npz")[0].projection == 1]
    loaded = [load_golden(GOLDEN / f"{c}.npz") for c in cases]
    runs = [M.Run(spec, ctx) for spec, _, _ in loaded]
    batch = M.Batch(runs)
    while batch.step(256):
        pass
    for c, (spec, meta, want), r in zip(cases, loaded, runs):
        t, dt, n = r.time()
        if init_only(meta):
            # the reference stops in the first cycle: so does the batched run
            code, cell = r.error()
            assert n <= 1 and (code & STOP_BITS[meta["reference_stop"]]), c
            continue
        assert n == int(meta["cycles"]), c
        assert t == float(meta["t"]), c
        for f in CELL_FIELDS + NODE_FIELDS + ["node_mass"]:
            assert_bitwise(f"{c}:{f}", get_field(r, f, spec.nbmat), want[f])


def test_batch_of_eucclhyd_reference_decks(M):
    """Every Eucclhyd golden deck with the remap (orders 1-3, one to three
    materials, PenteBorne variants, the conservative projection, the flux
    boundary, Noh, shock bubble, unit tests) in one batch: the Eucclhyd
    phases run on their own kernels, the sweeps on the shared ones, and each
    run matches the reference's final state (or stops where it stops)."""
    ctx = M.Context(0)
    cases = [c for c in golden_cases()
             if load_golden(GOLDEN / f"{c}.npz")[0].scheme == M.SCHEME_EUCCLHYD
             and load_golden(GOLDEN / f"{c}.npz")[0].projection == 1]
    assert len(cases) > 10
    loaded = [load_golden(GOLDEN / f"{c}.npz") for c in cases]
    runs = [M.Run(spec, ctx) for spec, _, _ in loaded]
    batch = M.Batch(runs)
    while batch.step(256):
        pass
    for c, (spec, meta, want), r in zip(cases, loaded, runs):
        t, dt, n = r.time()
        if init_only(meta):
            code, cell = r.error()
            assert n <= 1 and (code & STOP_BITS[meta["reference_stop"]]), c
            continue
        assert n == int(meta["cycles"]), c
        assert t == float(meta["t"]), c
        for f in fields_of(spec):
            assert_bitwise(f"{c}:{f}", get_field(r, f, spec.nbmat), want[f])


def test_batch_mixed_schemes_matches_plain(M):
    """VNR runs of the seeded mix and Eucclhyd reference decks in one batch,
    30 cycles: each run equals the same run advanced alone, bit for bit."""
    ctx = M.Context(0)
    vnr = [inst.spec(M) for inst in small_mix(6, seed=23)]
    euc = [load_golden(GOLDEN / f"{c}.npz")[0] for c in golden_cases()
           if load_golden(GOLDEN / f"{c}.npz")[0].scheme == M.SCHEME_EUCCLHYD
           and load_golden(GOLDEN / f"{c}.npz")[0].projection == 1
           and not init_only(load_golden(GOLDEN / f"{c}.npz")[1])][:6]
    specs = [x for pair in zip(vnr, euc) for x in pair]
    runs = [M.Run(s, ctx) for s in specs]
    M.Batch(runs).step(30)
    for s, rb in zip(specs, runs):
        alone = M.Run(s, ctx)
        alone.step(30)
        for f in fields_of(s):
            assert_bitwise(f"{s.scheme}:{s.nx}x{s.ny}:{f}", get_field(rb, f, s.nbmat),
                           get_field(alone, f, s.nbmat))
        assert rb.time() == alone.time() and rb.error() == alone.error()


def test_batch_membership_change(M):
    """The same context batches different run lists one after another; a
    run can leave a batch and continue alone."""
    ctx = M.Context(0)
    mix = small_mix(9, seed=3)
    specs = [inst.spec(M) for inst in mix]
    runs = [M.Run(s, ctx) for s in specs]
    ref = [M.Run(s, ctx) for s in specs]
    M.Batch(runs).step(10)
    M.Batch(runs[:5]).step(7)          # smaller list: same device block
    runs[5].step(7)                    # the others continue alone
    M.Batch(runs[6:]).step(7)
    M.Batch(list(reversed(runs))).step(23)
    for r in ref:
        r.step(40)
    for s, a, b in zip(specs, runs, ref):
        compare_runs(M, a, b, s.nbmat, f"{s.nx}x{s.ny}")


def test_batch_untuned_matches_tuned(M):
    ctx = M.Context(0)
    M.set_batch_tuning(ctx, False)
    mix = small_mix(8, seed=17)
    specs = [inst.spec(M) for inst in mix]
    a = [M.Run(s, ctx) for s in specs]
    M.Batch(a).step(40)
    assert not M.Batch(a).config()["tuned"]
    ctx2 = M.Context(0)
    b = [M.Run(s, ctx2) for s in specs]
    M.Batch(b).step(40)
    for s, x, y in zip(specs, a, b):
        compare_runs(M, x, y, s.nbmat, f"{s.nx}x{s.ny}")


def test_batch_and_server_refuse_runs_without_remap(M):
    """The batched and served forms advance runs with the remap: a
    Lagrange-only run is refused with a clear error (and the context stays
    usable); it runs on the plain path."""
    spec, _, _ = load_golden(GOLDEN / "SOD_X_Mono_mat_Lagrange_Vnr.npz")
    ctx = M.Context(0)
    run = M.Run(spec, ctx)
    with pytest.raises(RuntimeError, match="remap"):
        M.Batch([run], ctx).step(1)
    srv = M.Server(ctx)
    with pytest.raises(RuntimeError, match="remap"):
        srv.submit(spec)
    srv.stop(drain=False)
    assert not run.step(5)
    assert run.time()[2] == 5

