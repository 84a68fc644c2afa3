"""The allocation-free CFL time-step entry point against the normal path.

Callers that may not allocate device memory (their own pool owns it) pass
their buffers to hydro_vnr_dt_noalloc; its only scratch is a fixed array
inside the library.  Two calls in a row, at two successive states of a run,
must give exactly the dt the run itself computes for its next cycle
(hydro_run_step, then hydro_run_time).  This file is collected last.
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
    s.pseudo_centree, s.init_variant, s.max_cycles = 0, 1, 100
    return s


def test_noalloc_dt_matches_run():
    torch = pytest.importorskip("torch")
    import mahyco_gb300 as M
    from mahyco_gb300 import build
    build.build()
    L = M.lib()
    f = L.hydro_vnr_dt_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    nx, ny = 96, 80
    spec = _spec(M, nx, ny)
    ctx = M.Context(0)
    run = M.Run(spec, ctx)
    run.step(30)  # leave the initial dt ramp's first cycles
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for _ in range(2):
        t, dt_n, n = run.time()
        uv = run.fetch("node_velocity").reshape(-1, 2)
        u = torch.from_numpy(np.ascontiguousarray(uv[:, 0])).cuda()
        v = torch.from_numpy(np.ascontiguousarray(uv[:, 1])).cuda()
        c = torch.from_numpy(run.fetch("sound_speed")).cuda()
        torch.cuda.synchronize()
        rc = f(nx, ny, spec.dx, spec.dy, u.data_ptr(), v.data_ptr(),
               c.data_ptr(), dt_n, out.data_ptr(), None)
        assert rc == 0, L.hydro_last_error()
        torch.cuda.synchronize()
        got = float(out.item())
        run.step(1)  # the run computes the same dt at the start of its cycle
        want = run.time()[1]
        assert got == want, (got, want)
    # sizes beyond the fixed scratch are refused, nothing is launched
    rc = f(2048, 2048, 1.0 / 2048, 1.0 / 2048, u.data_ptr(), v.data_ptr(),
           c.data_ptr(), dt_n, out.data_ptr(), None)
    assert rc != 0 and b"scratch limit" in L.hydro_last_error()
