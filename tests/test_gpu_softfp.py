"""The integer-pipe binary64 operations on the GPU (hydro_softfp_check):
wherever the fast path applies, its result equals the GB300's own FP64
instruction bit for bit (the device form uses the FP32 approximate
reciprocal / reciprocal square root as its first estimate, unlike the host
form tested on the CPU)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OPS = {"mul": 0, "add": 1, "div": 2, "sqrt": 3, "sub": 4}


def _operands(rng, n):
    s = rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    f = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    mode = rng.integers(0, 5, n)
    e = np.where(mode == 0, rng.integers(1, 2047, n),
        np.where(mode == 1, rng.integers(983, 1063, n),
        np.where(mode == 2, rng.integers(0, 2048, n),
        np.where(mode == 3, rng.integers(1020, 1027, n),
                 np.where(rng.integers(0, 2, n) == 1, rng.integers(1, 5, n),
                          rng.integers(2043, 2047, n)))))).astype(np.uint64)
    k = (np.uint64(1) << rng.integers(0, 52, n).astype(np.uint64)) - np.uint64(1)
    few = np.where(rng.integers(0, 2, n) == 1, f & ~k, f | k)
    f = np.where(mode == 3, few, f)
    return s | (e << np.uint64(52)) | f


def _edge():
    base = [1.0, 1.5, 2.0, 3.0, 0.1, 1 / 3, 1e-300, 1e300, 2.0 ** -1022,
            np.finfo(np.float64).max, 1 + 2.0 ** -52, 2 - 2.0 ** -52, 0.0, 5e-324,
            1e-310, np.inf, np.nan, 2.0 ** -1000, 2.0 ** 1000]
    b = np.array(base, dtype=np.float64).view(np.uint64)
    vals = np.concatenate([b, b | np.uint64(1 << 63), b + np.uint64(1), b - np.uint64(1)])
    a, c = np.meshgrid(vals, vals)
    return a.ravel(), c.ravel()


@pytest.mark.parametrize("op", list(OPS))
def test_softfp_matches_fp64_instruction(op):
    torch = pytest.importorskip("torch")
    import mahyco_gb300 as M
    from mahyco_gb300 import build
    build.build()
    L = M.lib()
    rng = np.random.default_rng(7 + OPS[op])
    n = 1 << 22
    a = _operands(rng, n)
    b = _operands(rng, n)
    close = rng.integers(0, 7, n) == 0  # near-cancelling sums, close quotients
    mask = (np.uint64(1) << rng.integers(0, 53, n).astype(np.uint64)) - np.uint64(1)
    b = np.where(close, (a & ~np.uint64((1 << 52) - 1)) ^ (rng.integers(0, 2, n, dtype=np.uint64)
                                                       << np.uint64(63)) |
                 ((a & np.uint64((1 << 52) - 1)) ^ (rng.integers(0, 1 << 52, n, dtype=np.uint64)
                                                    & mask)), b)
    ea, eb = _edge()
    a = np.concatenate([a, ea])
    b = np.concatenate([b, eb])
    n = a.size
    da = torch.from_numpy(a.view(np.float64)).cuda()
    db = torch.from_numpy(b.view(np.float64)).cuda()
    soft = torch.empty_like(da)
    hw = torch.empty_like(da)
    fast = torch.empty(n, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    rc = L.hydro_softfp_check(OPS[op], da.data_ptr(), db.data_ptr(), soft.data_ptr(),
                              hw.data_ptr(), fast.data_ptr(), n, None)
    assert rc == 0, L.hydro_last_error()
    torch.cuda.synchronize()
    s = soft.cpu().numpy().view(np.uint64)
    h = hw.cpu().numpy().view(np.uint64)
    f = fast.cpu().numpy().astype(bool)
    assert f.sum() > n // 3, (op, int(f.sum()), n)
    bad = np.flatnonzero(f & (s != h))
    assert bad.size == 0, [(a[i].view(np.float64), b[i].view(np.float64),
                            s[i].view(np.float64), h[i].view(np.float64)) for i in bad[:5]]
    # the host's IEEE result agrees with the device instruction (normal cases)
    with np.errstate(all="ignore"):
        x, y = a.view(np.float64), b.view(np.float64)
        ref = {"mul": x * y, "add": x + y, "div": x / y, "sqrt": np.sqrt(x),
               "sub": x - y}[op].view(np.uint64)
    assert np.array_equal(ref[f], s[f])


def test_softfp_rates_measured():
    import mahyco_gb300 as M
    from mahyco_gb300 import build
    build.build()
    r = M.softfp_rates(0)
    for op, v in r.items():
        assert v["fp64_pipe"] > 0 and v["integer_pipe"] > 0, (op, v)
    print({op: round(v["integer_pipe"] / v["fp64_pipe"], 2) for op, v in r.items()})
