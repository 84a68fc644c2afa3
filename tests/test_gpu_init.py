"""The initial state built on the device (kernels/init.cu) equals the
oracle's host-side set-up (Vnr::simulate / Eucclhyd::simulate restated) bit
for bit, before any cycle: every golden deck's options, the extensions (VNR
Sedov, the mixed interface row, the advection step, the scaled triple point
with per-material exponents) and uneven mesh sizes."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, assert_bitwise, golden_cases, load_golden

pytestmark = pytest.mark.gpu

VNR_FIELDS = ["density", "pressure", "energy", "sound_speed", "pseudo", "divu",
              "cell_mass", "density_env", "energy_env", "pressure_env",
              "fracvol_env", "mass_fraction_env", "node_velocity", "node_mass"]
EUC_FIELDS = ["density", "energy", "cell_velocity", "density_env", "energy_env",
              "fracvol_env", "mass_fraction_env", "node_velocity"]


@pytest.fixture(scope="module")
def M():
    import mahyco_gb300
    from mahyco_gb300 import build
    build.build()
    return mahyco_gb300


def compare_initial(M, spec, tag):
    from oracle.port import PortRun
    run = M.Run(spec)
    ref = PortRun(spec)
    fields = EUC_FIELDS if spec.scheme == M.SCHEME_EUCCLHYD else VNR_FIELDS
    for f in fields:
        got, want = run.fetch(f), ref.fetch(f)
        if f.endswith("_env"):
            got = got.reshape(-1, 3)[:, :spec.nbmat]
            want = want.reshape(-1, 3)[:, :spec.nbmat]
        assert_bitwise(f"{tag}:{f}", got, want)
    assert run.time() == ref.time(), tag
    # the first cycle's time step (from the initial state's reduction)
    run.step(1)
    ref.step(1)
    assert run.time() == ref.time(), tag + " after one cycle"


@pytest.mark.parametrize("case", golden_cases())
def test_initial_state_of_golden_decks(M, port_lib, case):
    spec, _, _ = load_golden(GOLDEN / f"{case}.npz")
    compare_initial(M, spec, case)


@pytest.mark.parametrize("nx,ny", [(37, 23), (128, 40), (3, 301)])
def test_initial_state_uneven_meshes(M, port_lib, nx, ny):
    from mahyco_gb300.workloads import Instance
    for kind, sub in (("sod", "X"), ("sod", "Y"), ("sedov", None), ("advection", None)):
        inst = Instance(kind, nx, ny, 2 if kind != "sedov" else 1, "superBee", 5, sub)
        compare_initial(M, inst.spec(M), f"{kind}{sub or ''}-{nx}x{ny}")


def test_initial_state_mixed_row_and_triple_point(M, port_lib):
    s = M.default_spec()
    s.scheme, s.test_case, s.nbmat = M.SCHEME_VNR, 16, 2
    s.nx, s.ny, s.dx, s.dy = 64, 48, 1.0 / 64, 1.0 / 48
    s.final_time, s.dt_min = 0.2, 1e-12
    s.limiter, s.pb, s.limiter_pure = M.LIMITERS["superBee"], 1, M.LIMITERS["arithmeticG"]
    s.pseudo_centree, s.init_variant, s.max_cycles = 0, 1, 5
    compare_initial(M, s, "bisod-mixed-row")
    s.test_case, s.nx, s.ny = 15, 48, 64
    s.dx, s.dy = 1.0 / 48, 1.0 / 64
    compare_initial(M, s, "bisod-x-mixed-column")
    t = M.default_spec()
    t.scheme, t.test_case, t.nbmat = M.SCHEME_EUCCLHYD, 13, 3
    t.nx, t.ny, t.dx, t.dy = 112, 48, 7.0 / 112, 3.0 / 48
    for m, g in enumerate((1.5, 1.4, 1.5)):
        t.eos[m] = 101
        t.gamma[m] = g
    t.cfl, t.final_time, t.dt_min, t.space_order = 0.4, 100.0, 1e-12, 2
    t.projection_order, t.limiter, t.init_variant, t.max_cycles = 3, M.LIMITERS["superBee"], 3, 5
    compare_initial(M, t, "triple-point")


def test_initial_state_fetched_in_several_chunks(M, port_lib):
    """Fields larger than one pinned staging chunk (8 MiB), with sizes that
    leave a ragged last chunk, come back in the caller's layout: one, two
    and three planes per value, a material slot past the run's materials
    read as zero."""
    from mahyco_gb300.workloads import Instance
    import bench
    sod = Instance("sod", 1100, 1001, 2, "superBee", 5, "X").spec(M)
    compare_initial(M, sod, "sod-1100x1001")
    run = M.Run(sod)
    for f in ("fracvol_env", "density_env", "energy_env"):
        third = run.fetch(f).reshape(-1, 3)[:, 2]
        assert not np.any(third.view(np.uint64)), f
    tp = bench.triple_point_spec(M, 1030, 1010, cycles=5)
    compare_initial(M, tp, "triple-point-1030x1010")
