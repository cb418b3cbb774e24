"""Benchmark: paths/sec of the GB300 path tracker on the 10×10 dense-cubic total-degree
homotopy (59,049 paths), with the plain FP64 GPU tracker and the CPU oracle beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload dense|sparse|uneven|polyhedral]

A "step" is one batched tracking call over all paths of the workload. Prints one JSON line.
Under torchrun (N > 1) every rank tracks its own seeded instance (weak scaling) and rank 0
prints the aggregate. --impl reference times the reference algorithm on the host CPU: the
HomotopyContinuation.jl package itself needs Julia, which is not installed, so the CPU leg is
the C++ restatement in oracle/ (kind "port") on all host threads.
"""
from __future__ import annotations

import argparse
import ctypes as ct
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "homotopycontinuation.jl_gb300"))

METRIC = "paths/sec at ≤1e-10 rel endpoint err: learned vs plain step control, 1 GB300"
N_VARS, DEGREE = 10, 3
WORKLOAD = "total-degree homotopy, 10 dense cubics in 10 complex variables (286 monomials each), 59,049 paths"
WORKLOADS = {
    "dense": WORKLOAD,
    "sparse": "total-degree homotopy, 8 sparse polynomials in 8 complex variables (8 random monomials of degree "
              "<= 4 plus a constant each), 65,536 paths, most diverging (endgame-heavy)",
    "uneven": "2,000 independent dense instances in one launch, n uniform in 3..8, each equation degree uniform "
              "in {2,3}, all total-degree paths of every instance",
    "polyhedral": "polyhedral homotopy of the 8x8 sparse system of the sparse workload: mixed-volume many paths "
                  "(toric stage, then the coefficient homotopy with the endgame)",
    "slp": "total-degree homotopy of 8 products of three complex Gaussian affine forms in 8 variables, given as a "
           "straight-line program (NVRTC kernel), 6,561 paths; the term-table kernel on its expansion beside it",
}


# hc_options::lockstep of the timed launch (hc_last_stats)
LOCKSTEP_NAMES = {0: "none: each warp on its own", 1: "the CTA's warps step together",
                  2: "the warps of each SM sub-partition step together",
                  3: "the warps of each pair of SM sub-partitions step together"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--step-control", default="learned", choices=["plain", "learned"])
    p.add_argument("--cpu-sample", type=int, default=12288, help="paths of the CPU baseline sample")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--paths", type=int, default=0, help="track only the first N paths (profiling cases)")
    p.add_argument("--instances", type=int, default=2000, help="uneven workload: number of instances (profiling cases)")
    p.add_argument("--autotune", action="store_true",
                   help="uneven workload: tune the paths per CTA work unit for every n first")
    p.add_argument("--workload", default="dense", choices=list(WORKLOADS),
                   help="dense: the headline workload; sparse and uneven: the endgame-heavy and batched cases")
    return p.parse_args()


def workload(seed, kind="dense"):
    import hcgpu as hc

    if kind == "sparse":
        F, g = hc.sparse_random_system(8, 8, 4, seed=seed)
    else:
        F, g = hc.dense_random_system(N_VARS, DEGREE, seed=seed)
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    return H, S


def flop_model(stats, n, precision):
    """Algorithmic FP64 / FP32 flops of one call from the device counters and the program
    census (complex multiply 6, complex multiply-add 8, complex add 2 flops)."""
    M, Tv, Tj = stats["monomials"], stats["value_terms"], stats["jacobian_terms"]
    mono = 6 * M
    val = 8 * Tv + 14 * 2 * n
    jac = 8 * Tj + 14 * n * n
    lu = 8 * sum((n - k - 1) ** 2 for k in range(n)) + 6 * n * (n - 1) / 2 + 10 * n
    solve = 16 * n * n
    taylor_per_order = 6 * M * 4 + 16 * Tv  # series (≤4 products per monomial) + two row orders
    dd = 84 * (Tv + M)
    f64 = (stats["evals_jac"] * (mono + val) + stats["evals"] * (mono + val) + stats["evals_dd"] * dd)
    f32 = 0.0
    jac_lu = stats["evals_jac"] * jac + stats["lu"] * lu + stats["solves"] * solve
    tay = stats["taylor_orders"] / 2.0 * taylor_per_order
    if precision == "mixed":
        f32 += jac_lu + tay
        f64 += stats["taylor_fp64_redo"] * taylor_per_order
    else:
        f64 += jac_lu + tay
    return f64, f32


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                mhz.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(mhz)) if mhz else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(mhz)}


def flush_l2(buf):
    buf.zero_()


def cpu_baseline(H, S, sample, nthreads=0):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import hco

    cores = nthreads or os.cpu_count()
    idx = np.linspace(0, len(S) - 1, sample).astype(np.int64)
    t = time.perf_counter()
    res, xs, _, _ = hco.track(H.G.term_arrays(), H.F.term_arrays(), H.gamma, S[idx], nthreads=cores)
    dt = time.perf_counter() - t
    return {"value": sample / dt, "unit": "paths/s", "cores": cores, "kind": "port",
            "sample": f"{sample} of {len(S)} paths (evenly spaced indices) of the same homotopy, C++ FP64 "
                      f"restatement of the reference EndgameTracker on {cores} threads, {dt:.1f} s"}, idx, xs, res


def run_reference(args):
    """--impl reference: the reference algorithm on the host CPU (oracle port, all threads)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload == "uneven":
        print(json.dumps({"impl": "reference", "metric": METRIC, "unavailable": "the reference CPU arm is timed on "
                          "the single-system workloads only"}), flush=True)
        return
    if args.workload == "polyhedral":
        return run_reference_polyhedral(args)
    H, S = workload(args.seed, args.workload)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import hco

    hco.build()
    cores = os.cpu_count()
    sample = min(args.cpu_sample, len(S))
    idx = np.linspace(0, len(S) - 1, sample).astype(np.int64)
    St = S[idx]
    for _ in range(args.warmup):
        hco.track(H.G.term_arrays(), H.F.term_arrays(), H.gamma, St[: max(64, sample // 8)], nthreads=cores)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        hco.track(H.G.term_arrays(), H.F.term_arrays(), H.gamma, St, nthreads=cores)
        times.append(time.perf_counter() - t)
    ms = 1000 * float(np.mean(times))
    value = sample / (ms / 1000)
    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded complex Gaussian coefficients)",
        "impl": "reference",
        "config": {"workload": WORKLOADS[args.workload], "seed": args.seed, "sample_paths": sample},
        "cpu_baseline": {"value": value, "unit": "paths/s", "cores": cores, "kind": "port",
                         "sample": f"{sample} evenly spaced paths of {len(S)} per step; HomotopyContinuation.jl needs "
                                   f"Julia (not installed), so the C++ restatement of its tracker runs instead"},
        "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference_polyhedral(args):
    """--impl reference --workload polyhedral: the oracle's polyhedral tracker (both stages, C++
    restatement of the reference PolyhedralTracker) on all host threads, on an evenly spaced
    sample of the start solutions per step."""
    import hcgpu as hc
    from hcgpu import polyhedral_homotopy as ph

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import hco
    import polyhedral_oracle as po

    hco.build()
    F, _ = hc.sparse_random_system(8, 8, 4, seed=args.seed)
    T, S = ph.polyhedral(F, seed=args.seed + 1)
    cores = os.cpu_count()
    sample = min(args.cpu_sample, len(S))
    idx = np.linspace(0, len(S) - 1, sample).astype(np.int64)
    sub = ph.PolyhedralStartSolutions(S.supports, S.start_coefficients, S.lifting, S.cells,
                                      cell_of=S.cell_of[idx], x=S.x[idx])
    for _ in range(args.warmup):
        po.track(T, ph.PolyhedralStartSolutions(S.supports, S.start_coefficients, S.lifting, S.cells,
                                                cell_of=sub.cell_of[:64], x=sub.x[:64]), nthreads=cores)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        po.track(T, sub, nthreads=cores)
        times.append(time.perf_counter() - t)
    ms = 1000 * float(np.mean(times))
    value = sample / (ms / 1000)
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded complex Gaussian coefficients)",
        "impl": "reference",
        "config": {"workload": WORKLOADS["polyhedral"], "seed": args.seed, "sample_paths": sample, "paths": len(S)},
        "cpu_baseline": {"value": value, "unit": "paths/s", "cores": cores, "kind": "port",
                         "sample": f"{sample} evenly spaced start solutions of {len(S)} per step, both stages; "
                                   f"HomotopyContinuation.jl needs Julia (not installed), so the C++ restatement "
                                   f"of its tracker runs instead"},
        "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    import hcgpu as hc
    from hcgpu import _lib

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.workload == "uneven":
        return main_uneven(args, torch, hc, _lib, local)
    if args.workload == "polyhedral":
        return main_polyhedral(args, torch, hc, _lib, local)
    if args.workload == "slp":
        return main_slp(args, torch, hc, _lib, local)
    H, S = workload(args.seed + rank, args.workload)
    if args.paths:
        S = S[: args.paths]
    npaths, n = S.shape
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)  # a real stream: the kernel and its events share it
    torch.cuda.set_stream(stream)
    d_starts = torch.from_numpy(np.ascontiguousarray(S).view(np.float64).reshape(-1)).to(dev)
    d_res = torch.empty(npaths * _lib.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    d_sol = torch.empty(npaths * n * 2, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    L = _lib.load()

    def tracker(precision, step_control):
        to = hc.TrackerOptions(precision=precision, step_control=step_control)
        return hc.EndgameTracker(H, to)

    def device_call(T):
        rc = L.hc_track_device(T._h.h, npaths, ct.c_void_p(d_starts.data_ptr()), 1, 1.0, 0.0, 0.0, 0.0,
                               ct.c_void_p(d_res.data_ptr()), ct.c_void_p(d_sol.data_ptr()), None, None,
                               ct.c_void_p(stream.cuda_stream))
        _lib.check(rc, T._h.h)

    def timed(T, steps, warmup):
        for _ in range(warmup):
            device_call(T)
        torch.cuda.synchronize()
        times = []
        for _ in range(steps):
            flush_l2(flush)
            if dist:
                dist.barrier()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            h0 = time.perf_counter()
            e0.record(stream)
            device_call(T)
            e1.record(stream)
            torch.cuda.synchronize()
            host_ms = 1000 * (time.perf_counter() - h0)
            dev_ms = e0.elapsed_time(e1)
            if not (0.8 * host_ms <= dev_ms <= 1.05 * host_ms + 1.0):
                raise RuntimeError(f"device timing {dev_ms:.3f} ms disagrees with host timing {host_ms:.3f} ms")
            times.append(dev_ms)
        return times

    fp64_peak, fp32_peak = _lib.fma_peak()
    T = tracker(args.precision, args.step_control)
    with ClockSampler(local) as clk:
        times = timed(T, args.steps, args.warmup)
    stats = T.stats()
    res = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)
    sol = d_sol.cpu().numpy().view(np.complex128).reshape(npaths, n)
    ms = float(np.mean(times))
    ms_max = ms
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = float(t.item())
    value = world * npaths / (ms_max / 1000)

    # plain FP64 GPU tracker on the same paths (the ratio's denominator) and endpoint check
    T64 = tracker("fp64", "plain")
    t64 = timed(T64, 1, 1)
    res64 = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)
    sol64 = d_sol.cpu().numpy().view(np.complex128).reshape(npaths, n)
    both = (res["return_code"] == 1) & (res64["return_code"] == 1) & (res["singular"] == 0) & (res64["singular"] == 0)
    rel = np.abs(sol[both] - sol64[both]).max(1) / np.abs(sol64[both]).max(1)
    counts = lambda r: {"nonsingular": int(((r["return_code"] == 1) & (r["singular"] == 0)).sum()),
                        "singular": int(((r["return_code"] == 1) & (r["singular"] == 1)).sum()),
                        "at_infinity": int(np.isin(r["return_code"], [2, 3]).sum()),
                        "failed": int((~np.isin(r["return_code"], [1, 2, 3])).sum())}

    # end to end through the public host API: host arrays in, host results out
    e2e_steps = max(1, min(args.steps, 3))
    out_res = np.zeros(npaths, dtype=_lib.RESULT_DTYPE)
    out_sol = np.zeros((npaths, n), dtype=np.complex128)
    pinned = torch.from_numpy(np.ascontiguousarray(S).view(np.float64).reshape(-1)).pin_memory()
    starts_np = pinned.numpy()
    e2e_times = []
    for _ in range(e2e_steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = L.hc_track(T._h.h, npaths, starts_np.ctypes.data_as(ct.c_void_p), 1, 1.0, 0.0, 0.0, 0.0,
                        out_res.ctypes.data_as(ct.c_void_p), out_sol.ctypes.data_as(ct.c_void_p), None, None)
        _lib.check(rc, T._h.h)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = float(np.mean(e2e_times))
    retracked = int(T.stats()["paths_retracked"])
    if dist:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": world * npaths / e2e_s, "unit": "paths/s", "h2d_bytes_per_step": int(S.nbytes),
           "d2h_bytes_per_step": int(out_res.nbytes + out_sol.nbytes)}

    f64, f32 = flop_model(stats, n, args.precision)
    dur_s = ms / 1000
    ach64 = f64 / dur_s / 1e12
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu, idx, xo, ro = cpu_baseline(H, S, min(args.cpu_sample, npaths))
        okc = (ro["return_code"] == 1) & (res["return_code"][idx] == 1)
        rel_oracle = float((np.abs(sol[idx][okc] - xo[okc]).max(1) / np.abs(xo[okc]).max(1)).max()) if okc.any() else None
        codes_equal = bool((ro["return_code"] == res["return_code"][idx]).all())
    else:
        rel_oracle, codes_equal = None, None

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64+c128" if args.precision == "mixed" else "c128",
            "data": "synthetic (seeded complex Gaussian coefficients, N(0,1/2) re/im)",
            "config": {"workload": WORKLOADS[args.workload], "seed": args.seed, "paths_per_gpu": npaths, "n": n,
                       "precision": args.precision, "step_control": args.step_control,
                       "l2": "256 MiB buffer written between timed steps (inputs are smaller than L2)",
                       "parallelism": f"weak: one seeded instance per GPU x{world}",
                       "warps_per_cta": stats["warps_per_block"], "ctas": stats["blocks"],
                       "lockstep": LOCKSTEP_NAMES[int(stats["lockstep"])]},
            "e2e": e2e,
            "gpu_launches": args.steps,
            "clocks": clk.summary(),
            "roofline": {"bound": "fp64", "achieved": ach64, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": ach64 / fp64_peak, "traffic": None,
                         "peak_source": "measured FP64 FMA microbenchmark (hc_fma_peak) on this GPU",
                         "fp32_achieved": f32 / dur_s / 1e12, "fp32_peak": fp32_peak,
                         "flops_fp64_per_launch": f64, "flops_fp32_per_launch": f32},
            "cpu_baseline": cpu,
            "plain_fp64_gpu": {"value": npaths / (float(np.mean(t64)) / 1000), "unit": "paths/s",
                               "counts": counts(res64)},
            "speedup_vs_plain_fp64_gpu": (npaths / dur_s) / (npaths / (float(np.mean(t64)) / 1000)),
            "counts": counts(res),
            "counts_identical_to_fp64": counts(res) == counts(res64),
            "max_rel_endpoint_err_vs_fp64_gpu": float(rel.max()) if len(rel) else None,
            "paths_retracked_by_jump_check": retracked,
            "max_rel_endpoint_err_vs_oracle_sample": rel_oracle,
            "codes_identical_to_oracle_sample": codes_equal,
            "device_counters": {k: stats[k] for k in ["evals_jac", "evals", "evals_dd", "taylor_orders", "lu",
                                                     "solves", "taylor_fp64_redo", "paths_to_fp64",
                                                     "learned_proposals", "learned_rejected"]},
            "steps_per_path": float((res["accepted_steps"] + res["rejected_steps"]).mean()),
            "steps_per_path_plain_fp64": float((res64["accepted_steps"] + res64["rejected_steps"]).mean()),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main_uneven(args, torch, hc, _lib, local):
    """The batched workload: 2,000 uneven instances tracked by one persistent launch per step
    (hc_track_batch_device, recorded once in a CUDA graph), with the plain FP64 batch beside it."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        raise SystemExit("--workload uneven runs on one GPU")
    inst = hc.uneven_instances(args.instances, args.seed)
    Hs = [hc.total_degree_homotopy(F, g) for F, g in inst]
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    L = _lib.load()

    unit_paths, staging = None, None
    tune_s = 0.0
    if args.autotune:
        t = time.perf_counter()
        unit_paths, staging = hc.autotune(Hs, hc.TrackerOptions(precision=args.precision,
                                                                step_control=args.step_control),
                                          candidates=(2, 4, 8, 16, 32), sample=60)
        tune_s = time.perf_counter() - t

    def batch(precision, step_control):
        return hc.BatchTracker(Hs, hc.TrackerOptions(precision=precision, step_control=step_control),
                               unit_paths=unit_paths, staging=staging if precision == args.precision else None)

    B = batch(args.precision, args.step_control)
    S = B.start_solutions()
    d_starts = torch.from_numpy(S.view(np.float64)).to(dev)
    d_res = torch.empty(B.total_paths * _lib.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    d_sol = torch.empty(2 * B.total_elements, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def device_call(Bt):
        rc = L.hc_track_batch_device(Bt._h.h, ct.c_void_p(d_starts.data_ptr()), 1, ct.c_void_p(d_res.data_ptr()),
                                     ct.c_void_p(d_sol.data_ptr()), ct.c_void_p(stream.cuda_stream))
        _lib.check(rc, Bt._h.h)

    def timed(Bt, steps, warmup):
        for _ in range(warmup):
            device_call(Bt)
        torch.cuda.synchronize()
        out = []
        for _ in range(steps):
            flush_l2(flush)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            device_call(Bt)
            e1.record(stream)
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1))
        return out

    def results():
        r = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)
        return r, d_sol.cpu().numpy().view(np.complex128)

    def counts(r):
        rc = r["return_code"]
        return {"nonsingular": int(((rc == 1) & (r["singular"] == 0)).sum()),
                "singular": int(((rc == 1) & (r["singular"] == 1)).sum()),
                "at_infinity": int(np.isin(rc, [2, 3]).sum()), "failed": int((~np.isin(rc, [1, 2, 3])).sum())}

    with ClockSampler(local) as clk:
        times = timed(B, args.steps, args.warmup)
    stats = B.stats()
    res, sol = results()
    ms = float(np.mean(times))
    B64 = batch("fp64", "plain")
    t64 = timed(B64, 1, 1)
    res64, sol64 = results()
    nvec = np.repeat(B.n, B.npaths)
    off = np.concatenate([[0], np.cumsum(nvec)])[:-1]

    def max_err(r, x):
        ok = (r["return_code"] == 1) & (res64["return_code"] == 1) & (r["singular"] == 0) & (res64["singular"] == 0)
        e = 0.0
        for k in np.nonzero(ok)[0]:
            a, b = x[off[k]:off[k] + nvec[k]], sol64[off[k]:off[k] + nvec[k]]
            e = max(e, float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)))
        return e

    err_device = max_err(res, sol)
    # end to end through the host API (which also re-tracks jumped paths, see hc_track_batch)
    out_res = np.zeros(B.total_paths, dtype=_lib.RESULT_DTYPE)
    out_sol = np.zeros(B.total_elements, dtype=np.complex128)
    pinned = torch.from_numpy(S.view(np.float64)).pin_memory().numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _lib.check(L.hc_track_batch(B._h.h, pinned.ctypes.data_as(ct.c_void_p), 1, out_res.ctypes.data_as(ct.c_void_p),
                                out_sol.ctypes.data_as(ct.c_void_p)), B._h.h)
    e2e_s = time.perf_counter() - t0
    retracked = int(B.stats()["paths_retracked"])
    err = max_err(out_res, out_sol)
    # roofline: the flop model of each instance's program census, weighted by its paths (the
    # device counters are totals over the batch; an estimate, as paths of different instances
    # take different numbers of steps)
    from math import comb

    w = np.asarray(B.npaths, dtype=np.float64) / B.total_paths
    f64 = f32 = 0.0
    for wi, H in zip(w, Hs):
        nn, dmax = H.n, int(max(H.degrees))
        census = {"monomials": comb(nn + dmax, dmax),
                  "value_terms": sum(len(c) for c in H.F.coefficients) + 2 * nn,
                  "jacobian_terms": sum(int((e > 0).sum()) for e in H.F.exponents) + nn}
        a, b = flop_model({**stats, **census}, nn, args.precision)
        f64 += wi * a
        f32 += wi * b
    fp64_peak, fp32_peak = _lib.fma_peak()
    ach = f64 / (ms / 1000) / 1e12
    roofline = {"bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s", "frac": ach / fp64_peak,
                "traffic": None, "peak_source": "measured FP64 FMA microbenchmark (hc_fma_peak) on this GPU",
                "fp32_achieved": f32 / (ms / 1000) / 1e12, "fp32_peak": fp32_peak,
                "flops_fp64_per_launch": f64, "flops_fp32_per_launch": f32,
                "model": "per-instance program census (dense supports: C(n+d,d) monomials), weighted by paths"}
    # CPU baseline: the oracle on every 20th instance, all its paths
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import hco

        cores = os.cpu_count()
        pick = list(range(0, len(Hs), 20))
        npick = 0
        t = time.perf_counter()
        for i in pick:
            Si = hc.total_degree_start_solutions(Hs[i].degrees)
            hco.track(Hs[i].G.term_arrays(), Hs[i].F.term_arrays(), Hs[i].gamma, Si, nthreads=cores)
            npick += len(Si)
        dt = time.perf_counter() - t
        cpu = {"value": npick / dt, "unit": "paths/s", "cores": cores, "kind": "port",
               "sample": f"every 20th instance ({len(pick)} instances, {npick} paths), C++ FP64 restatement of the "
                         f"reference EndgameTracker on {cores} threads, {dt:.1f} s"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": B.total_paths / (ms / 1000), "unit": "paths/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64+c128" if args.precision == "mixed" else "c128",
            "data": "synthetic (seeded complex Gaussian coefficients, N(0,1/2) re/im)",
            "config": {"workload": WORKLOADS["uneven"], "seed": args.seed, "instances": len(Hs),
                       "paths": B.total_paths, "precision": args.precision, "step_control": args.step_control,
                       "ctas": stats["blocks"], "warps_per_cta": stats["warps_per_block"],
                       "lockstep": LOCKSTEP_NAMES[int(stats["lockstep"])],
                       "unit_paths": ({str(k): int(v) for k, v in unit_paths.items()} if unit_paths
                                      else "default: one path per warp of a CTA"),
                       "staging": ({str(k): v for k, v in staging.items()} if staging
                                   else "default: FP64 coefficients via L1/L2, rare FP64 areas in global"
                                   if args.precision == "mixed" else "shared"),
                       "autotune_seconds": tune_s,
                       "l2": "256 MiB buffer written between timed steps"},
            "e2e": {"value": B.total_paths / e2e_s, "unit": "paths/s", "h2d_bytes_per_step": int(S.nbytes),
                    "d2h_bytes_per_step": int(out_res.nbytes + out_sol.nbytes)},
            "gpu_launches": args.steps,
            "clocks": clk.summary(),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "plain_fp64_gpu": {"value": B.total_paths / (float(np.mean(t64)) / 1000), "unit": "paths/s",
                               "counts": counts(res64)},
            "speedup_vs_plain_fp64_gpu": float(np.mean(t64)) / ms,
            "counts": counts(out_res),
            "counts_identical_to_fp64": counts(out_res) == counts(res64),
            "codes_differing_from_fp64": int((out_res["return_code"] != res64["return_code"]).sum()),
            "max_rel_endpoint_err_vs_fp64_gpu": err,
            "paths_retracked_by_jump_check": retracked,
            "max_rel_endpoint_err_device_call_unchecked": err_device,
            "steps_per_path": float((res["accepted_steps"] + res["rejected_steps"]).mean()),
            "steps_per_path_plain_fp64": float((res64["accepted_steps"] + res64["rejected_steps"]).mean()),
        }
        print(json.dumps(line), flush=True)


def main_slp(args, torch, hc, _lib, local):
    """A structured system as a straight-line program (hc_set_slp: CUDA C from the program,
    compiled by NVRTC with the tracking kernel) against the term-table kernel on the same
    system expanded (165 monomials per equation); device-resident inputs, CUDA events."""
    from hcgpu import slp

    rank = int(os.environ.get("RANK", "0"))
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        raise SystemExit("--workload slp runs on one GPU")
    P, Fx = slp.products_of_linear_forms(8, 3, seed=args.seed)
    g = np.exp(2j * np.pi * 0.123)
    P.scaling = [float(np.max(np.abs(c))) for c in Fx.coefficients]
    Htab = hc.total_degree_homotopy(Fx, g)
    S = hc.total_degree_start_solutions(Htab.degrees)
    npaths, n = S.shape
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    d_starts = torch.from_numpy(np.ascontiguousarray(S).view(np.float64).reshape(-1)).to(dev)
    d_res = torch.empty(npaths * _lib.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    d_sol = torch.empty(npaths * n * 2, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    L = _lib.load()

    def call(T):
        _lib.check(L.hc_track_device(T._h.h, npaths, ct.c_void_p(d_starts.data_ptr()), 1, 1.0, 0.0, 0.0, 0.0,
                                     ct.c_void_p(d_res.data_ptr()), ct.c_void_p(d_sol.data_ptr()), None, None,
                                     ct.c_void_p(stream.cuda_stream)), T._h.h)

    def timed(T, steps, warmup):
        for _ in range(warmup):
            call(T)
        out = []
        for _ in range(steps):
            flush_l2(flush)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            call(T)
            e1.record(stream)
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1))
        res = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)
        return float(np.mean(out)), res, d_sol.cpu().numpy().view(np.complex128).reshape(npaths, n)

    to = hc.TrackerOptions(precision=args.precision, step_control=args.step_control)
    t = time.perf_counter()
    Ts = hc.EndgameTracker(slp.slp_homotopy(P, g), to)
    build_s = time.perf_counter() - t
    with ClockSampler(local) as clk:
        ms, rs, xs = timed(Ts, args.steps, args.warmup)
    Tt = hc.EndgameTracker(Htab, hc.TrackerOptions(precision=args.precision, step_control=args.step_control))
    ms_t, rt, xt = timed(Tt, args.steps, args.warmup)
    T64 = hc.EndgameTracker(Htab, hc.TrackerOptions())
    ms64, r64, x64 = timed(T64, 1, 1)
    ok = (rs["return_code"] == 1) & (rs["singular"] == 0) & (r64["return_code"] == 1) & (r64["singular"] == 0)
    err = float((np.abs(xs[ok] - x64[ok]).max(1) / np.abs(x64[ok]).max(1)).max()) if ok.any() else 0.0
    cpu = None
    if not args.no_cpu:
        cpu = cpu_baseline(Htab, S, min(args.cpu_sample, npaths))[0]
        cpu["sample"] += " (the expanded system)"
    if rank == 0:
        def counts(r):
            rc = r["return_code"]
            return {"nonsingular": int(((rc == 1) & (r["singular"] == 0)).sum()),
                    "singular": int(((rc == 1) & (r["singular"] == 1)).sum()),
                    "at_infinity": int(np.isin(rc, [2, 3]).sum()), "failed": int((~np.isin(rc, [1, 2, 3])).sum())}

        line = {
            "metric": METRIC, "value": npaths / (ms / 1000), "unit": "paths/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64+c128" if args.precision == "mixed" else "c128",
            "data": "synthetic (seeded complex Gaussian coefficients, N(0,1/2) re/im)",
            "config": {"workload": WORKLOADS["slp"], "seed": args.seed, "paths": npaths,
                       "program_instructions": len(P._tape.instr),
                       "expanded_terms_per_equation": len(Fx.coefficients[0]),
                       "nvrtc_build_seconds": build_s, "precision": args.precision, "step_control": args.step_control,
                       "l2": "256 MiB buffer written between timed steps"},
            "e2e": None,
            "gpu_launches": args.steps,
            "clocks": clk.summary(),
            "roofline": None,
            "cpu_baseline": cpu,
            "term_table_kernel": {"value": npaths / (ms_t / 1000), "unit": "paths/s", "counts": counts(rt)},
            "slp_vs_term_table": ms_t / ms,
            "counts": counts(rs), "counts_identical_to_fp64_table": counts(rs) == counts(r64),
            "codes_differing_from_fp64_table": int((rs["return_code"] != r64["return_code"]).sum()),
            "max_rel_endpoint_err_vs_fp64_table": err,
        }
        print(json.dumps(line), flush=True)


def main_polyhedral(args, torch, hc, _lib, local):
    """solve(F; start_system = :polyhedral) of the 8x8 sparse system: mixed cells and start
    solutions on the host (timed apart), then per step both tracking stages through the host
    API (hc_track_toric in FP64, then hc_track for the coefficient homotopy with the endgame in
    --precision / --step-control), with the all-FP64 plain run and the total-degree solve of the
    same system beside it."""
    from hcgpu import polyhedral_homotopy as ph

    rank = int(os.environ.get("RANK", "0"))
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        raise SystemExit("--workload polyhedral runs on one GPU")
    F, g = hc.sparse_random_system(8, 8, 4, seed=args.seed)
    t = time.perf_counter()
    T64, S = ph.polyhedral(F, seed=args.seed + 1)
    prep_s = time.perf_counter() - t
    npaths = len(S)
    T = ph.PolyhedralTracker(T64.supports, T64.start_coeffs, T64.target_coeffs, T64.lifting, T64.cells, T64.n,
                             hc.TrackerOptions(precision=args.precision, step_control=args.step_control))

    def timed(Tr, steps, warmup):
        for _ in range(warmup):
            Tr.track_arrays(S)
        out = []
        for _ in range(steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rs_ = Tr.track_arrays(S)
            out.append(time.perf_counter() - t0)
        return out, rs_

    with ClockSampler(local) as clk:
        times, rs = timed(T, args.steps, args.warmup)
    ms = 1000 * float(np.mean(times))
    t64, rs64 = timed(T64, 1, 1)

    def counts(rr):
        return {"nonsingular": sum(r.is_success() and not r.is_singular() for r in rr),
                "singular": sum(r.is_success() and r.is_singular() for r in rr),
                "failed": sum(not r.is_success() for r in rr)}

    err = 0.0
    for a_, b_ in zip(rs, rs64):
        if a_.is_success() and b_.is_success() and not a_.is_singular() and not b_.is_singular():
            err = max(err, float(np.abs(a_.solution - b_.solution).max() / max(np.abs(b_.solution).max(), 1e-300)))
    # roofline: the flop model over the three launches of the last timed step (toric stage and
    # its restart in FP64, the coefficient homotopy in --precision), from each handle's counters
    f64 = f32 = 0.0
    for key, hh in T._handles.items():
        a, b = flop_model(hh.stats(), T.n, args.precision if key == "generic" else "fp64")
        f64 += a
        f32 += b
    fp64_peak, fp32_peak = _lib.fma_peak()
    ach = f64 / (ms / 1000) / 1e12
    roofline = {"bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s", "frac": ach / fp64_peak,
                "traffic": None, "peak_source": "measured FP64 FMA microbenchmark (hc_fma_peak) on this GPU",
                "fp32_achieved": f32 / (ms / 1000) / 1e12, "fp32_peak": fp32_peak,
                "flops_fp64_per_step": f64, "flops_fp32_per_step": f32,
                "model": "program census x device counters of the toric, restart and coefficient launches; time "
                         "includes the host API's copies"}
    # total degree on the same system (plain FP64)
    H = hc.total_degree_homotopy(F, g)
    S2 = hc.total_degree_start_solutions(H.degrees)
    E = hc.EndgameTracker(H, hc.TrackerOptions())
    E.track_arrays(S2[:4096])
    torch.cuda.synchronize()
    t = time.perf_counter()
    r2 = E.track_batch(S2)
    td_s = time.perf_counter() - t
    # CPU baseline: the oracle's polyhedral tracker on an evenly spaced sample of the paths
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import polyhedral_oracle as po

        sample = min(args.cpu_sample, npaths)
        idx = np.linspace(0, npaths - 1, sample).astype(np.int64)
        sub = ph.PolyhedralStartSolutions(S.supports, S.start_coefficients, S.lifting, S.cells,
                                          cell_of=S.cell_of[idx], x=S.x[idx])
        cores = os.cpu_count()
        t = time.perf_counter()
        ocodes, ox, _ = po.track(T64, sub, nthreads=cores)
        dt = time.perf_counter() - t
        agree = int(sum((ocodes[j] == 1) == rs64[k].is_success() for j, k in enumerate(idx)))
        cpu = {"value": sample / dt, "unit": "paths/s", "cores": cores, "kind": "port",
               "sample": f"{sample} of {npaths} paths (evenly spaced), C++ FP64 restatement of the reference "
                         f"PolyhedralTracker on {cores} threads, {dt:.1f} s; success flags agree with the FP64 GPU "
                         f"run on {agree}"}
    if rank == 0:
        codes = [r.return_code for r in rs]
        line = {
            "metric": METRIC, "value": npaths / (ms / 1000), "unit": "paths/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64+c128" if args.precision == "mixed" else "c128",
            "data": "synthetic (seeded complex Gaussian coefficients, N(0,1/2) re/im)",
            "config": {"workload": WORKLOADS["polyhedral"], "seed": args.seed, "paths": npaths,
                       "mixed_cells": len(T.cells), "host_preparation_seconds": prep_s,
                       "timing": "host API per step (starts copied in, results copied out): value and e2e coincide",
                       "precision": f"toric stage fp64, coefficient homotopy {args.precision}",
                       "step_control": f"toric stage plain, coefficient homotopy {args.step_control}"},
            "e2e": {"value": npaths / (ms / 1000), "unit": "paths/s",
                    "h2d_bytes_per_step": int(S.x.nbytes * 2), "d2h_bytes_per_step": int(S.x.nbytes * 2)},
            "gpu_launches": 3,
            "clocks": clk.summary(),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "counts": counts(rs), "codes": {c: codes.count(c) for c in set(codes)},
            "plain_fp64_gpu": {"value": npaths / float(np.mean(t64)), "unit": "paths/s", "counts": counts(rs64)},
            "speedup_vs_plain_fp64_gpu": float(np.mean(t64)) / (ms / 1000),
            "counts_identical_to_fp64": counts(rs) == counts(rs64),
            "max_rel_endpoint_err_vs_fp64_gpu": err,
            "total_degree_same_system": {"paths": len(S2), "seconds": td_s,
                                         "nonsingular": sum(r.is_success() and not r.is_singular() for r in r2)},
            "speedup_vs_total_degree_gpu": td_s / (ms / 1000),
        }
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
