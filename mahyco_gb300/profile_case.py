"""Small fixed workload for profiler captures (ncu), launched through the C
ABI: the benchmark's bi-material Sod case on an n x n mesh (VNR), or the
triple point on an (7n/3) x n mesh (Eucclhyd, --scheme euc), a few cycles.
A developed flow is captured in two runs: one advances the case and writes a
checkpoint (--advance N --save PATH), the profiled one restores it and runs
the cycles to capture (--restore PATH), so that the capture holds only those.
python -m mahyco_gb300.profile_case [--mesh 1024] [--cycles 3] [--scheme vnr|euc]
    [--advance N --save PATH | --restore PATH]"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--mesh", type=int, default=1024)
    ap.add_argument("--cycles", type=int, default=3)
    ap.add_argument("--scheme", default="vnr", choices=["vnr", "euc"])
    ap.add_argument("--advance", type=int, default=0)
    ap.add_argument("--save", default=None)
    ap.add_argument("--restore", default=None)
    a = ap.parse_args()
    import mahyco_gb300 as M
    from bench import triple_point_spec, workload_spec
    total = a.advance + a.cycles
    if a.scheme == "euc":
        spec = triple_point_spec(M, 7 * a.mesh // 3, a.mesh, total)
    else:
        spec = workload_spec(M, a.mesh, total)
    if a.restore:
        run = M.Run.restore(a.restore)
        run.step(a.cycles)
    else:
        run = M.Run(spec)
        run.step(a.advance if a.save else a.cycles)
        if a.save:
            run.checkpoint(a.save)
    code, _ = run.error()
    print(f"profile_case: {a.scheme} {spec.nx}x{spec.ny}, {run.time()[2]} cycles, "
          f"error word {code}")


if __name__ == "__main__":
    main()
