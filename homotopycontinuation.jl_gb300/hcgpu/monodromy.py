"""Monodromy solving (src/monodromy.jl) on the batched GPU tracker.

Start from one or more solutions x of F(x; p) = 0 at a base parameter p, move the parameters
around loops p → p₁ → p₂ → p (p₁, p₂ drawn from the complex normal distribution, as the
reference's ``independent_normal`` sampler does, src/monodromy.jl:54-75) and collect the new
distinct endpoints at p. The reference tracks one loop edge at a time; here a *round* runs
``loops_per_round`` loops side by side, and every edge of a round is ONE batched launch over
all loops' paths (hc_set_batch / hc_track_batch). Stopping rules as in the reference:
``target_solutions_count`` reached, or ``max_loops_no_progress`` loops in a row without a
new solution, or ``timeout`` seconds.

``find_start_pair`` (src/monodromy.jl: find_start_pair) works when the parameters enter the
coefficients linearly, which every ParametricSystem does: for a random x, F(x; p) = 0 is a
linear system in p.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from .batch import BatchTracker
from .parameters import ParameterHomotopy, ParametricSystem
from .tracking import EndgameOptions, TrackerOptions


def _cnormal(rng, size):
    return (rng.standard_normal(size) + 1j * rng.standard_normal(size)) / np.sqrt(2)


def find_start_pair(F: ParametricSystem, seed: Optional[int] = None, max_tries: int = 100):
    """A pair (x, p) with F(x; p) = 0: x random complex normal, p the minimum-norm solution of
    the linear system F(x; p) = 0 plus a random element of its null space. None if the
    parameters cannot absorb the equations (the system in p is inconsistent)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    for _ in range(max_tries):
        x = _cnormal(rng, F.n)
        A = np.zeros((F.nequations, F.nparams), dtype=np.complex128)
        b = np.zeros(F.nequations, dtype=np.complex128)
        for i, (e, c0, C) in enumerate(zip(F.exponents, F.c0, F.C)):
            m = np.prod(x[None, :] ** e, axis=1)
            A[i] = m @ C
            b[i] = m @ c0
        p, *_ = np.linalg.lstsq(A, -b, rcond=None)
        if np.abs(A @ p + b).max() > 1e-10 * max(1.0, np.abs(b).max()):
            continue
        # a generic point of the affine solution space
        _, sv, vh = np.linalg.svd(A)
        rank = int((sv > 1e-12 * sv.max()).sum()) if sv.size else 0
        N = vh[rank:].conj().T
        if N.shape[1]:
            p = p + N @ _cnormal(rng, N.shape[1])
        if np.abs(F(p).evaluate(x)).max() <= 1e-9 * max(1.0, np.abs(p).max()):
            return x, p
    return None


class _UniquePoints:
    """Distinct points up to rtol (relative to max(‖x‖∞, 1)), indexed by a scaled coordinate."""

    def __init__(self, rtol=1e-8):
        self.rtol = rtol
        self.points: list = []
        self.keys: list = []

    def add(self, x) -> bool:
        x = np.asarray(x, dtype=np.complex128)
        s = max(np.abs(x).max(), 1.0)
        key = x[0].real / s
        lo = np.searchsorted(self.keys, key - 4 * self.rtol)
        hi = np.searchsorted(self.keys, key + 4 * self.rtol, side="right")
        for j in range(lo, hi):
            y = self.points[j]
            if np.abs(x - y).max() <= self.rtol * max(s, np.abs(y).max(), 1.0):
                return False
        j = int(np.searchsorted(self.keys, key))
        self.keys.insert(j, key)
        self.points.insert(j, x)
        return True

    def __len__(self):
        return len(self.points)


@dataclass
class MonodromyResult:
    """src/monodromy.jl MonodromyResult: the distinct solutions at the base parameters."""

    solutions: list
    parameters: np.ndarray
    returncode: str  # "success" (target count reached) | "heuristic_stop" | "timeout"
    loops: int = 0
    rounds: int = 0
    tracked_paths: int = 0
    seconds: float = 0.0
    history: list = field(default_factory=list)

    def nsolutions(self) -> int:
        return len(self.solutions)

    def is_success(self) -> bool:
        return self.returncode == "success"

    def is_heuristic_stop(self) -> bool:
        return self.returncode == "heuristic_stop"


def monodromy_solve(F: ParametricSystem, sols=None, p=None, *, seed: Optional[int] = None,
                    target_solutions_count: Optional[int] = None, max_loops_no_progress: int = 5,
                    timeout: Optional[float] = None, loops_per_round: int = 4,
                    tracker_options: Optional[TrackerOptions] = None, unique_points_rtol: float = 1e-8,
                    check_startsolutions: bool = True) -> MonodromyResult:
    """monodromy_solve(F, [sols, p]; options...) (src/monodromy.jl:632-720)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if sols is None or p is None:
        pair = find_start_pair(F, seed=None if seed is None else seed + 1)
        if pair is None:
            raise ValueError("cannot compute a start pair (x, p): pass solutions and parameters explicitly")
        x0, p = pair
        sols = [x0]
    p = np.asarray(p, dtype=np.complex128).reshape(-1)
    to = tracker_options or TrackerOptions()
    eo = EndgameOptions()
    U = _UniquePoints(unique_points_rtol)
    for s in sols:
        s = np.asarray(s, dtype=np.complex128)
        if check_startsolutions and np.abs(F(p).evaluate(s)).max() > 1e-8 * max(1.0, np.abs(s).max()):
            continue
        U.add(s)
    if len(U) == 0:
        raise ValueError("no valid start solution")
    t0 = time.time()
    no_progress = 0
    loops = rounds = tracked = 0
    history = []
    code = "heuristic_stop"
    B = None  # one batch tracker (handle, buffers, step model) for every edge
    while True:
        if target_solutions_count is not None and len(U) >= target_solutions_count:
            code = "success"
            break
        if no_progress >= max_loops_no_progress:
            break
        if timeout is not None and time.time() - t0 > timeout:
            code = "timeout"
            break
        k = loops_per_round
        S = np.array(U.points)
        legs = [[p, _cnormal(rng, F.nparams), _cnormal(rng, F.nparams), p] for _ in range(k)]
        current = [S.copy() for _ in range(k)]
        for e in range(3):
            alive = [i for i in range(k) if len(current[i])]
            if not alive:
                break
            Hs = [ParameterHomotopy(F, legs[i][e], legs[i][e + 1]) for i in alive]
            if B is None:
                B = BatchTracker(Hs, to, eo, npaths=[len(current[i]) for i in alive])
            else:
                B.set_homotopies(Hs, npaths=[len(current[i]) for i in alive])
            res, sol = B.track_arrays(np.concatenate([current[i].reshape(-1) for i in alive]))
            tracked += B.total_paths
            for (r, x), i in zip(B.split(res, sol), alive):
                ok = (r["return_code"] == 1) & (r["singular"] == 0)
                current[i] = x[ok]
        new = 0
        for i in range(k):
            loops += 1
            found = sum(U.add(x) for x in current[i])
            new += found
            no_progress = 0 if found else no_progress + 1
            if target_solutions_count is not None and len(U) >= target_solutions_count:
                break
        rounds += 1
        history.append(dict(round=rounds, solutions=len(U), new=new, tracked=tracked))
    return MonodromyResult(solutions=[np.array(x) for x in U.points], parameters=p, returncode=code,
                           loops=loops, rounds=rounds, tracked_paths=tracked, seconds=time.time() - t0,
                           history=history)


def main(argv=None):
    """python -m hcgpu.monodromy [--n 7] [--degree 2] [--seed 0]: monodromy over the coefficient
    space of a seeded dense system from one start pair, against its total-degree solve."""
    import argparse
    import json

    from .systems import dense_random_system
    from .tracking import solve

    ap = argparse.ArgumentParser(description=main.__doc__.split("\n")[0])
    ap.add_argument("--n", type=int, default=7)
    ap.add_argument("--degree", type=int, default=2)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--loops-per-round", type=int, default=4)
    a = ap.parse_args(argv)
    F0, _ = dense_random_system(a.n, a.degree, seed=a.seed)
    Fp = ParametricSystem.coefficient_parameters(F0)
    bezout = a.degree ** a.n
    R = monodromy_solve(Fp, seed=a.seed, target_solutions_count=bezout, max_loops_no_progress=10,
                        loops_per_round=a.loops_per_round)
    t = time.time()
    T = solve(Fp(R.parameters))
    td = time.time() - t
    print(json.dumps({"system": f"{a.n} dense polynomials of degree {a.degree}, coefficients as parameters",
                      "bezout": bezout, "monodromy_solutions": R.nsolutions(), "returncode": R.returncode,
                      "rounds": R.rounds, "loops": R.loops, "tracked_paths": R.tracked_paths,
                      "monodromy_seconds": R.seconds, "total_degree_solutions": T.nsolutions(),
                      "total_degree_seconds": td}))


if __name__ == "__main__":
    main()
