"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: long-running CPU check")


def load_golden(path: Path):
    import mahyco_gb300 as M
    z = np.load(path)
    spec = M.HydroSpec()
    for k, v in json.loads(str(z["spec"])).items():
        if isinstance(v, list):
            arr = getattr(spec, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(spec, k, v)
    meta = json.loads(str(z["meta"]))
    fields = {k: z[k] for k in z.files if k not in ("spec", "meta")}
    return spec, meta, fields


def golden_cases():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


# fields compared per case; *_env fields keep only the nbmat live columns
CELL_FIELDS = ["density", "pressure", "energy", "sound_speed", "pseudo", "divu",
               "cell_mass", "density_env", "energy_env", "pressure_env",
               "fracvol_env", "mass_fraction_env"]
NODE_FIELDS = ["node_velocity"]
EUC_FIELDS = ["density", "pressure", "energy", "sound_speed", "cell_velocity",
              "density_env", "energy_env", "fracvol_env", "mass_fraction_env",
              "node_velocity"]


# fields of an initial-state fixture (harness --init-only): a Eucclhyd run's
# pressure and sound speed are first formed by its first cycle
EUC_INIT_FIELDS = ["density", "energy", "cell_velocity", "density_env", "energy_env",
                   "fracvol_env", "mass_fraction_env", "node_velocity"]
# error word bit of the way the reference stops in the first cycle
STOP_BITS = {"nan": 1, "energy": 2, "dt": 4}


def init_only(meta) -> bool:
    """An initial-state fixture: the reference stops in the first cycle."""
    return meta.get("init_only") == "1"


def init_fields_of(spec):
    return EUC_INIT_FIELDS if spec.scheme == 2000 else CELL_FIELDS + NODE_FIELDS + ["node_mass"]


def check_first_cycle_stop(run, meta):
    """The run, stepped from its initial state, stops in the first cycle
    with the error the reference stops on (and at the cell it names)."""
    done = run.step(3)
    code, cell = run.error()
    assert done and (code & STOP_BITS[meta["reference_stop"]]), (code, meta["reference_stop"])
    if int(meta["reference_stop_cell"]) >= 0:
        assert cell == int(meta["reference_stop_cell"]), (cell, meta["reference_stop_cell"])
    assert run.time()[2] <= 1


def fields_of(spec):
    """Fields a fixture of this scheme holds (all compared bit for bit)."""
    if spec.scheme == 2000:  # Eucclhyd
        return EUC_FIELDS
    return CELL_FIELDS + NODE_FIELDS + ["node_mass"]


def get_field(run, name, nbmat):
    a = run.fetch(name)
    if name.endswith("_env"):
        a = a.reshape(-1, 3)[:, :nbmat]
    return a


def assert_bitwise(name, got, want):
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape, (name, got.shape, want.shape)
    if not np.array_equal(got, want, equal_nan=True):
        d = np.abs(got - want)
        i = int(np.nanargmax(d))
        raise AssertionError(
            f"{name}: {int(np.sum(got != want))} values differ, max |diff| "
            f"{np.nanmax(d):.3e} at {i}: got {got.flat[i]!r} want {want.flat[i]!r}")


@pytest.fixture(scope="session")
def port_lib():
    from oracle import port
    port.build()
    return port
