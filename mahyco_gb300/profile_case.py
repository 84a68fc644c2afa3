"""Small fixed workload for profiler captures (ncu): the benchmark's
bi-material Sod case on an n x n mesh, a few cycles, launched through the C
ABI.  python -m mahyco_gb300.profile_case [--mesh 1024] [--cycles 3]"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--mesh", type=int, default=1024)
    ap.add_argument("--cycles", type=int, default=3)
    a = ap.parse_args()
    import mahyco_gb300 as M
    from bench import workload_spec
    run = M.Run(workload_spec(M, a.mesh, a.cycles))
    run.step(a.cycles)
    code, _ = run.error()
    print(f"profile_case: {a.mesh}^2, {run.time()[2]} cycles, error word {code}")


if __name__ == "__main__":
    main()
