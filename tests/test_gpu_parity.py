"""CUDA path against the reference (golden vectors) and the C restatement.

Bit-exact: every golden case (the reference's own VNR decks with remap, the
200x10 Sod workload, a 64x64 bi-material Sod with a mixed interface row) must
reproduce the reference's final state bit for bit, through the C ABI.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import (CELL_FIELDS, GOLDEN, NODE_FIELDS, assert_bitwise,
                      check_first_cycle_stop, fields_of, get_field, golden_cases,
                      init_fields_of, init_only, load_golden)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    import mahyco_gb300
    from mahyco_gb300 import build
    build.build()
    return mahyco_gb300


@pytest.fixture(scope="module")
def ctx(M):
    return M.Context(0)


@pytest.mark.parametrize("case", golden_cases())
def test_gpu_matches_reference(case, M, ctx):
    spec, meta, want = load_golden(GOLDEN / f"{case}.npz")
    run = M.Run(spec, ctx)
    if init_only(meta):
        # the reference stops in the first cycle: its initial state, then
        # the same stop through the error word
        assert run.time() == (0.0, float(meta["dt"]), 0)
        for f in init_fields_of(spec):
            assert_bitwise(f"{case}:{f}", get_field(run, f, spec.nbmat), want[f])
        check_first_cycle_stop(run, meta)
        return
    run.simulate(chunk=256)
    t, dt, n = run.time()
    assert n == int(meta["cycles"])
    assert t == float(meta["t"])
    for f in fields_of(spec):
        assert_bitwise(f"{case}:{f}", get_field(run, f, spec.nbmat), want[f])
    assert run.error()[0] & ~M.ERR_NEGATIVE == 0


def _bisod(M, n, cycles, pb=True, limiter="superBee", dual=0):
    s = M.default_spec()
    s.scheme, s.test_case, s.nbmat = M.SCHEME_VNR, 16, 2
    s.nx = s.ny = n
    s.dx = s.dy = 1.0 / n
    s.final_time, s.output_time, s.dt_init, s.dt_min = 0.2, 1e-2, 1e-4, 1e-12
    s.projection, s.projection_order = 1, 2
    s.limiter = M.LIMITERS[limiter]
    s.pb, s.pb_mixte, s.limiter_pure, s.pb_complet = int(pb), 0, M.LIMITERS["arithmeticG"], 0
    s.pseudo_centree, s.dual_mass_flux = 0, dual
    s.init_variant = 1
    s.max_cycles = cycles
    return s


@pytest.mark.parametrize("n,cycles,pb,lim,dual", [
    (256, 120, True, "superBee", 0),
    (256, 120, False, "minmod", 0),
    (192, 100, True, "superBee", 2),
    (160, 100, True, "minmod", 1),
])
def test_gpu_matches_port_larger(n, cycles, pb, lim, dual, M, ctx, port_lib):
    spec = _bisod(M, n, cycles, pb, lim, dual)
    g = M.Run(spec, ctx)
    g.simulate()
    c = port_lib.PortRun(spec)
    c.simulate()
    assert g.time() == c.time()
    for f in CELL_FIELDS + NODE_FIELDS:
        assert_bitwise(f, get_field(g, f, spec.nbmat), get_field(c, f, spec.nbmat))


def vnr_totals(run, spec):
    """Total mass, x / y momentum and total energy of a VNR state, from the
    fetched fields (exactly rounded sums): cell masses rho * V on the Euler
    mesh, nodal momentum m_p u_p, internal energy rho e V plus the nodal
    kinetic energy m_p |u_p|^2 / 2."""
    V = spec.dx * spec.dy
    rho, e = run.fetch("density"), run.fetch("energy")
    mp = run.fetch("node_mass")
    u = run.fetch("node_velocity").reshape(-1, 2)
    return {"mass": math.fsum(rho * V),
            "momentum_x": math.fsum(mp * u[:, 0]),
            "momentum_y": math.fsum(mp * u[:, 1]),
            "energy": math.fsum(rho * e * V) + math.fsum(0.5 * mp * (u[:, 0] ** 2 + u[:, 1] ** 2)),
            # momentum scale: the whole mass moving at the largest sound speed
            "momentum_scale": math.fsum(mp) * float(np.max(run.fetch("sound_speed")))}


def test_gpu_config2_full_size_matches_port(M, ctx, port_lib):
    """The large single-instance workload exactly as benchmarked (bi-material
    Sod Y on 2048^2 with the 50/50 mixed row, VNR, order 2, superBee +
    PenteBorne pure, A1 dual flux, 200 cycles): every cell and node field
    bit-identical to the C restatement, and the conservation totals.

    Mass is conserved to 1e-13 relative.  Momentum is not a conserved
    quantity of this problem (the walls push on the fluid: the initial
    pressure jump between the bottom and top walls accelerates it upwards);
    x-momentum, zero by the mirror symmetry in x, stays within 1e-13 of the
    momentum scale (total mass times the largest sound speed).  Total energy
    is not conserved exactly by the reference's staggered scheme (its remap
    of the nodal kinetic energy is not conservative: the C restatement, bit
    for bit the reference, drifts by 5e-8 over 200 cycles on 256^2 and by
    2e-5 over 1400), so the energy totals are checked equal to the port's."""
    import bench
    spec = bench.workload_spec(M, 2048, 200)
    run = M.Run(spec, ctx)
    t0 = vnr_totals(run, spec)
    run.simulate()
    assert run.time()[2] == 200
    ref = port_lib.PortRun(spec)
    ref.simulate()
    assert run.time() == ref.time()
    for f in CELL_FIELDS + NODE_FIELDS + ["node_mass"]:
        assert_bitwise(f, get_field(run, f, spec.nbmat), get_field(ref, f, spec.nbmat))
    t1, tr = vnr_totals(run, spec), vnr_totals(ref, spec)
    assert t1 == tr
    assert abs(t1["mass"] - t0["mass"]) <= 1e-13 * t0["mass"]
    assert abs(t1["momentum_x"]) <= 1e-13 * t1["momentum_scale"]
    rho = run.fetch("density")
    assert np.all(np.isfinite(rho)) and rho.min() > 0
    assert run.error()[0] & ~M.ERR_NEGATIVE == 0


def test_gpu_developed_flow_matches_port(M, ctx, port_lib):
    """The benchmark deck on 256^2 run well past the initial dt ramp, until
    the waves cross most of the mesh (most nodes moving, so the exact
    at-rest shortcuts are taken almost nowhere): every field bit-identical to
    the C restatement, mass conserved to 1e-13 relative."""
    import bench
    spec = bench.workload_spec(M, 256, 1400)
    run = M.Run(spec, ctx)
    t0 = vnr_totals(run, spec)
    run.simulate()
    ref = port_lib.PortRun(spec)
    ref.simulate()
    assert run.time() == ref.time()
    u = run.fetch("node_velocity").reshape(-1, 2)
    moving = float(np.mean((u[:, 0] != 0) | (u[:, 1] != 0)))
    assert moving > 0.6, moving
    for f in CELL_FIELDS + NODE_FIELDS + ["node_mass"]:
        assert_bitwise(f, get_field(run, f, spec.nbmat), get_field(ref, f, spec.nbmat))
    t1 = vnr_totals(run, spec)
    assert t1 == vnr_totals(ref, spec)
    assert abs(t1["mass"] - t0["mass"]) <= 1e-13 * t0["mass"]
    assert abs(t1["momentum_x"]) <= 1e-13 * t1["momentum_scale"]


def test_gpu_error_word_instead_of_abort(M, ctx):
    """The reference exits when |e_mat| exceeds 5 (vnr_remap/PhaseLagrange.cc
    :358-369); the GPU path records the error in the device error word, stops
    the run, and the context stays usable."""
    spec, meta, _ = load_golden(GOLDEN / "SOD_X_Mono_mat_Minmod_vnr_o2.npz")
    spec.energy_limit = 1.0  # initial energies are 2.5 / 2.0
    run = M.Run(spec, ctx)
    done = run.step(5)
    code, cell = run.error()
    assert done and (code & M.ERR_ENERGY) and cell >= 0
    assert run.time()[2] == 1
    ok = M.Run(load_golden(GOLDEN / "SOD_X_Mono_mat_Minmod_vnr_o2.npz")[0], ctx)
    ok.step(3)
    assert ok.error()[0] == 0


def triple_point(M, nx, ny, cycles, order=3):
    """The three-material triple point on [0,7]x[0,3] (Eucclhyd, superBee
    with PenteBorne mixte, arithmeticG in pure cells, CFL 0.4, exponents
    1.5 / 1.4 / 1.5, regions x <= 1 and y <= 1.5 scaled to the domain)."""
    s = M.default_spec()
    s.scheme, s.test_case, s.nbmat = M.SCHEME_EUCCLHYD, 13, 3
    s.nx, s.ny = nx, ny
    s.dx, s.dy = 7.0 / nx, 3.0 / ny
    for m, g in enumerate((1.5, 1.4, 1.5)):
        s.eos[m] = 101
        s.gamma[m] = g
    s.gamma_scalar = 1.4
    s.cfl = 0.4
    s.final_time, s.dt_min, s.space_order = 100.0, 1e-12, 2
    s.projection, s.projection_order = 1, order
    s.limiter = M.LIMITERS["superBee"]
    s.pb, s.pb_mixte, s.limiter_pure, s.pb_complet = 1, 1, M.LIMITERS["arithmeticG"], 0
    s.init_variant = 3
    s.max_cycles = cycles
    return s


@pytest.mark.parametrize("order,pb,complet", [(3, 0, 0), (2, 1, 0), (2, 1, 1), (3, 1, 0)])
def test_gpu_triple_point_matches_port(order, pb, complet, M, ctx, port_lib):
    """Order 3 with PenteBorne reproduces the reference's arithmetic, which
    takes the order-3 face value as an integrated flux: the state turns
    negative and the run stops with a NaN error in the second cycle, on the
    GPU as in the reference."""
    from conftest import EUC_FIELDS
    spec = triple_point(M, 224, 96, 60, order)
    spec.pb, spec.pb_mixte, spec.pb_complet = pb, pb, complet
    g = M.Run(spec, ctx)
    g.simulate()
    c = port_lib.PortRun(spec)
    c.simulate()
    assert g.time() == c.time()
    assert g.error() == c.error()
    for f in EUC_FIELDS:
        assert_bitwise(f, get_field(g, f, spec.nbmat), get_field(c, f, spec.nbmat))


def test_gpu_triple_point_full_size_matches_port(M, ctx, port_lib):
    """1792x768 triple point (the Eucclhyd workload: order-3 projection,
    superBee), 8 cycles: bit-identical to the C restatement at full size;
    total mass moves by less than 1e-11 relative (the remap's volume
    normalisation is not exactly conservative in the reference either)."""
    from conftest import EUC_FIELDS
    spec = triple_point(M, 1792, 768, 8)
    spec.pb = spec.pb_mixte = 0
    run = M.Run(spec, ctx)
    vol = 7.0 * 3.0 / (1792 * 768)
    m0 = run.fetch("density").sum() * vol
    run.simulate()
    ref = port_lib.PortRun(spec)
    ref.simulate()
    assert run.time() == ref.time()
    for f in EUC_FIELDS:
        assert_bitwise(f, get_field(run, f, spec.nbmat), get_field(ref, f, spec.nbmat))
    m1 = run.fetch("density").sum() * vol
    assert abs(m1 - m0) <= 1e-11 * m0
    assert run.error()[0] & ~M.ERR_NEGATIVE == 0
    assert run.time()[2] == 8


def euc_totals(run, spec):
    """Total mass, momentum and energy of a Eucclhyd state from the fetched
    cell-centred fields (exactly rounded sums over rho V, rho u V and
    rho (e + |u|^2 / 2) V on the Euler mesh)."""
    V = spec.dx * spec.dy
    rho, e = run.fetch("density"), run.fetch("energy")
    u = run.fetch("cell_velocity").reshape(-1, 2)
    m = rho * V
    return {"mass": math.fsum(m), "momentum_x": math.fsum(m * u[:, 0]),
            "momentum_y": math.fsum(m * u[:, 1]),
            "energy": math.fsum(m * (e + 0.5 * (u[:, 0] ** 2 + u[:, 1] ** 2)))}


def test_gpu_triple_point_conservation(M, ctx, port_lib):
    """224x96 triple point, 300 cycles (order-3 projection, superBee): the
    mass, momentum and energy totals equal the C restatement's (bit for bit
    the reference).  The reference conserves none of them to 1e-13 here:
    the walls push on the fluid (momentum), the kinetic energy is remapped
    without the conservative correction, and the C restatement itself moves
    the mass rho V by -2.6e-5 and the total energy by -6.3e-4 over these
    cycles; so the check is equality with the port, with bounds just above
    those drifts."""
    spec = triple_point(M, 224, 96, 300)
    spec.pb = spec.pb_mixte = 0
    run = M.Run(spec, ctx)
    t0 = euc_totals(run, spec)
    run.simulate()
    ref = port_lib.PortRun(spec)
    ref.simulate()
    assert run.time() == ref.time()
    t1 = euc_totals(run, spec)
    assert t1 == euc_totals(ref, spec)
    assert abs(t1["mass"] - t0["mass"]) <= 1e-4 * t0["mass"]
    assert abs(t1["energy"] - t0["energy"]) <= 1e-3 * t0["energy"]


@pytest.mark.parametrize("case", ["UNIT_vnr_init", "BIUNIT_vnr_init"])
def test_gpu_left_flux_boundary_matches_port(case, M, ctx, port_lib):
    """The VNR unit tests, whose remap takes a flux through the left side
    (remap/BoundaryFluxes.cc, leftFluxBC of vnr_remap/Init.cc:65-93), run
    for 300 cycles with the |e| > 5 abort switched off (energy_limit 0: the
    reference stops on it in the first cycle, which the golden test pins):
    bit-identical to the C restatement, the inflow visible in the mass."""
    spec, _, _ = load_golden(GOLDEN / f"{case}.npz")
    spec.energy_limit = 0.0
    spec.max_cycles = 300
    spec.final_time = 10.0
    g = M.Run(spec, ctx)
    m0 = math.fsum(g.fetch("density")) * spec.dx * spec.dy
    g.simulate()
    c = port_lib.PortRun(spec)
    c.simulate()
    assert g.time() == c.time() and g.time()[2] == 300
    assert g.error() == c.error()
    for f in CELL_FIELDS + NODE_FIELDS + ["node_mass"]:
        assert_bitwise(f"{case}:{f}", get_field(g, f, spec.nbmat), get_field(c, f, spec.nbmat))
    m1 = math.fsum(g.fetch("density")) * spec.dx * spec.dy
    assert m1 != m0


@pytest.mark.parametrize("order,pb", [(2, 0), (2, 1), (3, 0)])
def test_gpu_shock_bubble_larger_matches_port(order, pb, M, ctx, port_lib):
    """The shock on a helium bubble on the reference deck's own 520x64 mesh
    (0.00125 spacing), 150 cycles: the right side's inflow through the
    remap's boundary flux, bit-identical to the C restatement."""
    spec, _, _ = load_golden(GOLDEN / "SHOCK_BUBBLE_MinMod_o2.npz")
    spec.nx, spec.ny, spec.dx, spec.dy = 520, 64, 0.00125, 0.00125
    spec.projection_order, spec.pb = order, pb
    spec.limiter = M.LIMITERS["superBee"]
    spec.max_cycles = 150
    g = M.Run(spec, ctx)
    g.simulate()
    c = port_lib.PortRun(spec)
    c.simulate()
    assert g.time() == c.time()
    assert g.error() == c.error()
    for f in fields_of(spec):
        assert_bitwise(f, get_field(g, f, spec.nbmat), get_field(c, f, spec.nbmat))


@pytest.mark.parametrize("case,centred", [("SOD_X_bi_mat_Lagrange_Vnr", 0),
                                          ("SOD_Y_Mono_mat_Lagrange_Vnr_Qcentree", 1)])
def test_gpu_lagrange_only_larger_matches_port(case, centred, M, ctx, port_lib):
    """VNR without the remap (the Lagrange phase alone, the mesh moving) on
    a mesh eight times the reference deck's, 400 cycles: every field and the
    node positions bit-identical to the C restatement, compared both in the
    middle of the run and at its end (pseudo_centree as the deck has it)."""
    spec, _, _ = load_golden(GOLDEN / f"{case}.npz")
    assert spec.projection == 0 and spec.pseudo_centree == centred
    spec.nx, spec.ny = spec.nx * 2 if spec.nx > spec.ny else spec.nx * 4, \
        spec.ny * 4 if spec.nx > spec.ny else spec.ny * 2
    spec.dx, spec.dy = (1.0 / spec.nx, 0.1 / spec.ny) if spec.nx > spec.ny else \
        (0.1 / spec.nx, 1.0 / spec.ny)
    spec.max_cycles = 400
    g = M.Run(spec, ctx)
    c = port_lib.PortRun(spec)
    g.step(250)
    c.step(250)
    assert g.time() == c.time()
    for f in CELL_FIELDS + NODE_FIELDS + ["node_coord"]:
        assert_bitwise(f"{case}@250:{f}", get_field(g, f, spec.nbmat), get_field(c, f, spec.nbmat))
    g.simulate()
    c.simulate()
    assert g.time() == c.time()
    for f in CELL_FIELDS + NODE_FIELDS + ["node_mass"]:
        assert_bitwise(f"{case}:{f}", get_field(g, f, spec.nbmat), get_field(c, f, spec.nbmat))
    assert g.error()[0] & ~M.ERR_NEGATIVE == 0
