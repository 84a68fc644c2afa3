"""Small fixed workload for profiler captures (ncu), launched through the C
ABI: the benchmark's bi-material Sod case on an n x n mesh (VNR), or the
triple point on an (7n/3) x n mesh (Eucclhyd, --scheme euc), a few cycles.
python -m mahyco_gb300.profile_case [--mesh 1024] [--cycles 3] [--scheme vnr|euc]"""
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
    a = ap.parse_args()
    import mahyco_gb300 as M
    from bench import triple_point_spec, workload_spec
    if a.scheme == "euc":
        spec = triple_point_spec(M, 7 * a.mesh // 3, a.mesh, a.cycles)
    else:
        spec = workload_spec(M, a.mesh, a.cycles)
    run = M.Run(spec)
    run.step(a.cycles)
    code, _ = run.error()
    print(f"profile_case: {a.scheme} {spec.nx}x{spec.ny}, {run.time()[2]} cycles, "
          f"error word {code}")


if __name__ == "__main__":
    main()
