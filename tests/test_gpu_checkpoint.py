"""Checkpoint / restart (hydro_run_checkpoint, hydro_run_restore): a run
restored from a checkpoint continues bit for bit as the original, for both
schemes, across processes and after the run has ended; damaged or foreign
files are rejected."""
from __future__ import annotations

import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

from conftest import CELL_FIELDS, EUC_FIELDS, NODE_FIELDS, assert_bitwise, get_field

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def M():
    import mahyco_gb300
    from mahyco_gb300 import build
    build.build()
    return mahyco_gb300


def bisod(M, n=64):
    s = M.default_spec()
    s.scheme, s.test_case, s.nbmat = M.SCHEME_VNR, 16, 2
    s.nx, s.ny, s.dx, s.dy = n, n - 16, 1.0 / n, 1.0 / (n - 16)
    s.final_time, s.dt_min = 0.2, 1e-12
    s.limiter, s.pb, s.limiter_pure = M.LIMITERS["superBee"], 1, M.LIMITERS["arithmeticG"]
    s.pseudo_centree, s.init_variant, s.max_cycles = 0, 1, 70
    return s


def triple_point(M):
    """Three-material triple point (Eucclhyd, order-3 remap without
    PenteBorne, exponents 1.5 / 1.4 / 1.5, CFL 0.4) on 112 x 48 cells."""
    s = M.default_spec()
    s.scheme, s.test_case, s.nbmat = M.SCHEME_EUCCLHYD, 13, 3
    s.nx, s.ny = 112, 48
    s.dx, s.dy = 7.0 / 112, 3.0 / 48
    for m, g in enumerate((1.5, 1.4, 1.5)):
        s.eos[m] = 101
        s.gamma[m] = g
    s.gamma_scalar, s.cfl = 1.4, 0.4
    s.final_time, s.dt_min, s.space_order = 100.0, 1e-12, 2
    s.projection, s.projection_order = 1, 3
    s.limiter, s.pb = M.LIMITERS["superBee"], 0
    s.init_variant, s.max_cycles = 3, 60
    return s


def fields(M, spec):
    if spec.scheme == M.SCHEME_EUCCLHYD:
        return EUC_FIELDS + ["VelocityX", "VelocityY", "Pressure"]
    return CELL_FIELDS + NODE_FIELDS + ["node_mass"]


def compare(M, a, b, spec, tag):
    for f in fields(M, spec):
        assert_bitwise(f"{tag}:{f}", get_field(a, f, spec.nbmat), get_field(b, f, spec.nbmat))
    assert a.time() == b.time(), tag
    assert a.error() == b.error(), tag


@pytest.mark.parametrize("case", ["vnr", "euc"])
def test_restore_continues_bit_for_bit(M, case, tmp_path):
    spec = bisod(M) if case == "vnr" else triple_point(M)
    ref = M.Run(spec)
    ref.step(23)
    ck = tmp_path / "run.ckpt"
    ref.checkpoint(ck)
    ref.step(30)
    back = M.Run.restore(ck)
    assert back.time()[2] == 23
    back.step(30)
    compare(M, ref, back, spec, case)
    # the original can go on after writing the checkpoint too
    plain = M.Run(spec)
    plain.step(53)
    compare(M, plain, ref, spec, case + "-uninterrupted")


def test_restore_in_another_process(M, tmp_path):
    spec = bisod(M, 96)
    ref = M.Run(spec)
    ref.step(17)
    ck = tmp_path / "a.ckpt"
    ref.checkpoint(ck)
    ref.simulate()
    out = tmp_path / "after.npz"
    code = textwrap.dedent(f"""
        import sys, numpy as np
        sys.path.insert(0, {str(ROOT)!r})
        import mahyco_gb300 as M
        r = M.Run.restore({str(ck)!r})
        r.simulate()
        t, dt, n = r.time()
        np.savez({str(out)!r}, density=r.fetch("density"), energy=r.fetch("energy"),
                 node_velocity=r.fetch("node_velocity"), t=t, n=n)
    """)
    subprocess.run([sys.executable, "-c", code], check=True, timeout=300)
    got = np.load(out)
    for f in ("density", "energy", "node_velocity"):
        assert_bitwise(f, got[f], ref.fetch(f))
    t, _, n = ref.time()
    assert float(got["t"]) == t and int(got["n"]) == n


def test_restore_of_finished_run_stays_finished(M, tmp_path):
    spec = bisod(M)
    spec.max_cycles = 12
    r = M.Run(spec)
    r.simulate()
    ck = tmp_path / "done.ckpt"
    r.checkpoint(ck)
    b = M.Run.restore(ck)
    assert b.step(5)  # done at once
    assert b.time() == r.time()


def test_damaged_or_foreign_files_are_rejected(M, tmp_path):
    spec = bisod(M)
    r = M.Run(spec)
    r.step(3)
    ck = tmp_path / "x.ckpt"
    r.checkpoint(ck)
    data = bytearray(ck.read_bytes())
    bad = tmp_path / "flip.ckpt"
    flip = bytearray(data)
    flip[len(flip) // 2] ^= 0x40
    bad.write_bytes(bytes(flip))
    with pytest.raises(RuntimeError, match="corrupted"):
        M.Run.restore(bad)
    # one option byte changed (the limiter id, after the 64-byte header):
    # the options carry their own hash, so the run does not resume with
    # another scheme
    opt = tmp_path / "option.ckpt"
    flip = bytearray(data)
    flip[64 + M.HydroSpec.limiter.offset] ^= 0x01
    opt.write_bytes(bytes(flip))
    with pytest.raises(RuntimeError, match="options corrupted"):
        M.Run.restore(opt)
    short = tmp_path / "short.ckpt"
    short.write_bytes(bytes(data[: len(data) - 4096]))
    with pytest.raises(RuntimeError, match="truncated"):
        M.Run.restore(short)
    other = tmp_path / "other.ckpt"
    other.write_bytes(b"not a checkpoint" * 8)
    with pytest.raises(RuntimeError, match="not a hydro checkpoint"):
        M.Run.restore(other)
    with pytest.raises(RuntimeError, match="cannot open"):
        M.Run.restore(tmp_path / "missing.ckpt")
    # the context is still usable after the rejections
    again = M.Run.restore(ck)
    again.step(2)
    r.step(2)
    compare(M, r, again, spec, "after-rejections")
