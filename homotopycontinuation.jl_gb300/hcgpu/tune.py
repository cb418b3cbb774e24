"""The batch launch-plan autotuner from the command line: prints, for every system size n of
the uneven workload, the milliseconds per launch of each (paths per unit, staging) pair that
hc_autotune_batch measured, and the plan it chose.

    python -m hcgpu.tune --instances 2000 --seed 0 --precision mixed --step-control learned
"""
from __future__ import annotations

import argparse
import time

from .batch import autotune
from .systems import total_degree_homotopy, uneven_instances
from .tracking import TrackerOptions


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m hcgpu.tune")
    ap.add_argument("--instances", type=int, default=2000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--step-control", default="learned", choices=["plain", "learned"])
    ap.add_argument("--sample", type=int, default=60, help="instances of each n that are timed")
    ap.add_argument("--repeats", type=int, default=2, help="timed launches per candidate (after one warm-up)")
    ap.add_argument("--candidates", default="2,4,8,16,32", help="paths per work unit")
    a = ap.parse_args(argv)
    Hs = [total_degree_homotopy(F, g) for F, g in uneven_instances(a.instances, a.seed)]
    opts = TrackerOptions(precision=a.precision, step_control=a.step_control)
    t = time.perf_counter()
    unit, staging = autotune(Hs, opts, tuple(int(c) for c in a.candidates.split(",")), sample=a.sample,
                             repeats=a.repeats, verbose=True)
    print(f"chosen in {time.perf_counter() - t:.1f} s: unit_paths {unit}, staging {staging}")


if __name__ == "__main__":
    main()
