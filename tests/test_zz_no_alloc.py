"""The allocation-free CFL time-step entry point against the normal path.

Callers that may not allocate device memory (their own pool owns it) pass
their buffers to hydro_vnr_dt_noalloc; its only scratch is a fixed array
inside the library.  Two calls in a row, at two successive states of a run,
must give exactly the dt the run itself computes for its next cycle
(hydro_run_step, then hydro_run_time), on two mesh shapes, one of them the
largest the scratch accepts.  The states are taken after the initial dt
ramp, so the minimum over the cells (not the 1.05 * dt_n growth cap)
decides the value.  This file is collected last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spec(M, nx, ny):
    s = M.default_spec()
    s.scheme, s.test_case, s.nbmat = M.SCHEME_VNR, 16, 2
    s.nx, s.ny, s.dx, s.dy = nx, ny, 1.0 / nx, 1.0 / ny
    s.final_time, s.dt_min = 0.2, 1e-12
    s.limiter, s.pb, s.limiter_pure = M.LIMITERS["superBee"], 1, M.LIMITERS["arithmeticG"]
    s.pseudo_centree, s.init_variant, s.max_cycles = 0, 1, 2000
    return s


def _entry(M):
    from mahyco_gb300 import build
    build.build()
    L = M.lib()
    f = L.hydro_vnr_dt_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return L, f


def _call(torch, L, f, nx, ny, dx, dy, u, v, c, dt_n):
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    du, dv, dc = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (u, v, c))
    torch.cuda.synchronize()
    rc = f(nx, ny, dx, dy, du.data_ptr(), dv.data_ptr(), dc.data_ptr(), dt_n,
           out.data_ptr(), None)
    assert rc == 0, L.hydro_last_error()
    torch.cuda.synchronize()
    return float(out.item())


def _candidates(nx, ny, dx, dy, u, v, c):
    """Per-cell CFL candidates with the kernel's (the reference's) operation
    order, in numpy float64 (every step an IEEE operation)."""
    i, j = np.divmod(np.arange(nx * ny), nx)
    fi, fj = i.astype(np.float64), j.astype(np.float64)
    X = [(dx * fj, dy * fi), (dx * (fj + 1), dy * fi),
         (dx * (fj + 1), dy * (fi + 1)), (dx * fj, dy * (fi + 1))]
    xc0 = 0.0 + X[0][0]
    xc1 = 0.0 + X[0][1]
    for k in range(1, 4):
        xc0 = xc0 + X[k][0]
        xc1 = xc1 + X[k][1]
    xc0, xc1 = 0.25 * xc0, 0.25 * xc1
    vs = np.zeros(nx * ny)
    for k in range(4):
        km, kp = (k + 3) & 3, (k + 1) & 3
        x2a, x2b = 0.5 * (X[km][0] + X[k][0]), 0.5 * (X[km][1] + X[k][1])
        x4a, x4b = 0.5 * (X[kp][0] + X[k][0]), 0.5 * (X[kp][1] + X[k][1])
        c12 = xc0 * x2b - xc1 * x2a
        c23 = x2a * X[k][1] - x2b * X[k][0]
        c34 = X[k][0] * x4b - X[k][1] * x4a
        c41 = x4a * xc1 - x4b * xc0
        vs = vs + 0.5 * (((c12 + c23) + c34) + c41)
    n0 = i * (nx + 1) + j
    uc = np.zeros(nx * ny)
    for nd in (n0, n0 + 1, n0 + nx + 2, n0 + nx + 1):
        uc = uc + np.sqrt(u[nd] * u[nd] + v[nd] * v[nd]) * 0.25
    with np.errstate(invalid="ignore", divide="ignore"):
        return (0.05 * np.sqrt(vs)) / (uc + c)


def _want(cand, dt_n):
    ok = cand[~np.isnan(cand)]
    red = ok.min() if ok.size else np.finfo(np.float64).max
    cap = 1.05 * dt_n
    return cap if cap < red else red


@pytest.mark.parametrize("nx,ny", [(96, 80), (1024, 1024)])
def test_noalloc_dt_matches_run(nx, ny):
    torch = pytest.importorskip("torch")
    import mahyco_gb300 as M
    L, f = _entry(M)
    spec = _spec(M, nx, ny)
    ctx = M.Context(0)
    run = M.Run(spec, ctx)
    run.step(400)  # past the initial dt ramp (dt_0 = 1e-6 of the CFL step, x1.05 per cycle)
    decided_by_cells = 0
    for _ in range(2):  # two calls in a row, two successive states
        t, dt_n, n = run.time()
        uv = run.fetch("node_velocity").reshape(-1, 2)
        c = run.fetch("sound_speed")
        got = _call(torch, L, f, nx, ny, spec.dx, spec.dy, uv[:, 0], uv[:, 1], c, dt_n)
        run.step(1)  # the run computes the same dt at the start of its cycle
        want = run.time()[1]
        assert got == want, (got, want)
        decided_by_cells += want < 1.05 * dt_n
    assert decided_by_cells == 2
    run.close()
    ctx.close()


def test_noalloc_dt_reduction_edges():
    torch = pytest.importorskip("torch")
    import mahyco_gb300 as M
    L, f = _entry(M)
    nx = ny = 1024  # exactly the largest mesh the scratch takes
    dx = dy = 1.0 / 1024
    rng = np.random.default_rng(11)
    nn = (nx + 1) * (ny + 1)
    u, v = rng.uniform(-1, 1, nn), rng.uniform(-1, 1, nn)
    c = rng.uniform(0.5, 2.0, nx * ny)
    # the minimum planted in the last cell, far from block 0
    last = nx * ny - 1
    i, j = divmod(last, nx)
    n0 = i * (nx + 1) + j
    for nd in (n0, n0 + 1, n0 + nx + 2, n0 + nx + 1):
        u[nd] = 50.0
    cand = _candidates(nx, ny, dx, dy, u, v, c)
    assert int(np.nanargmin(cand)) == last
    for dt_n in (1.0, 1e-9):  # the minimum decides, then the growth cap
        got = _call(torch, L, f, nx, ny, dx, dy, u, v, c, dt_n)
        assert got == _want(cand, dt_n), (got, _want(cand, dt_n))
    # NaN candidates are skipped (std::min keeps its first argument)
    c2 = c.copy()
    c2[::3] = np.nan
    cand2 = _candidates(nx, ny, dx, dy, u, v, c2)
    got = _call(torch, L, f, nx, ny, dx, dy, u, v, c2, 1.0)
    assert got == _want(cand2, 1.0)
    # no valid candidate at all: the reduction's DBL_MAX start, then the cap
    c3 = np.full(nx * ny, np.nan)
    got = _call(torch, L, f, nx, ny, dx, dy, u, v, c3, 2.0)
    assert got == 1.05 * 2.0
    # one row more than the scratch holds is refused before any launch
    buf = torch.zeros((nx + 2) * (ny + 2), dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    rc = f(nx, ny + 1, dx, dy, p, p, p, 1.0, p, None)
    assert rc != 0 and b"scratch limit" in L.hydro_last_error()
    assert float(buf[0].item()) == 0.0
