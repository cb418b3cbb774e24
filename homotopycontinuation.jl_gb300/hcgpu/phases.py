"""Where the tracker's cycles go: builds a profiling copy of libhcgpu.so with the phase cycle
counters compiled in (-DHC_PHASE_CLOCKS), tracks a workload and prints, per tracker phase,
its share of the per-path cycles and its cycles per step.

    python -m hcgpu.phases [--paths 8192] [--modes mixed_learned,mixed_plain,fp64_plain]

Workload: the total-degree homotopy of 10 dense cubics in 10 variables (seed 0), the first
``--paths`` start solutions. The counters are per warp (lane 0, clock64) and inclusive: a
solve includes the LU factorization it triggers, Newton includes its evaluations. The
reference's analogue is the per-step ``debug`` trace of src/tracker.jl:855-888.
"""
from __future__ import annotations

import argparse
import os
import time

PHASE_BUILD = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "_build_phase")


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--paths", type=int, default=8192)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--modes", default="mixed_learned,mixed_plain,fp64_plain")
    a = ap.parse_args(argv)
    from . import _build

    lib = _build.build(defines=("HC_PHASE_CLOCKS",), build_dir=PHASE_BUILD)
    os.environ["HCGPU_LIB"] = lib
    import torch

    from . import learn
    from .systems import dense_random_system, total_degree_homotopy, total_degree_start_solutions
    from .tracking import EndgameTracker, TrackerOptions, _Handle

    F, g = dense_random_system(10, 3, seed=a.seed)
    H = total_degree_homotopy(F, g)
    S = total_degree_start_solutions(H.degrees)[: a.paths]
    opts = {
        "mixed_learned": lambda: TrackerOptions(precision="mixed", step_control="learned",
                                                step_model=learn.default_model()),
        "mixed_plain": lambda: TrackerOptions(precision="mixed"),
        "fp64_plain": lambda: TrackerOptions(precision="fp64"),
        "fp64_learned": lambda: TrackerOptions(precision="fp64", step_control="learned",
                                               step_model=learn.default_model()),
    }
    names = [k for k in _Handle.STAT_NAMES if k.startswith("clk_")]
    for mode in a.modes.split(","):
        T = EndgameTracker(H, opts[mode]())
        T.track_arrays(S[:64])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r, _, _, _ = T.track_arrays(S)
        dt = time.perf_counter() - t0
        st = T.stats()
        steps = float((r["accepted_steps"] + r["rejected_steps"]).sum())
        run = st["clk_run"]
        if run == 0:
            raise RuntimeError("phase counters are zero: the profiling library was not loaded")
        print(f"{mode}: {len(S) / dt:.0f} paths/s (profiling build), {steps / len(S):.1f} steps/path, "
              f"{run / steps:.3e} cycles/step per warp")
        for k in names:
            print(f"   {k[4:]:10s} {100 * st[k] / run:6.2f}%  {st[k] / steps:12.0f} cycles/step")


if __name__ == "__main__":
    main()
