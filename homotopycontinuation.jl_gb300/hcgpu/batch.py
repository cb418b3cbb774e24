"""Batches of independent total-degree homotopies tracked in one GPU launch.

The reference solves independent systems one ``solve(F_i)`` at a time (src/solve.jl:447-526),
each running its own ``threaded_solve`` loop over paths (src/solve.jl:628-709). Here all
instances of a batch share one persistent launch (``hc_set_batch`` / ``hc_track_batch``): CTAs
take work units (instance, path range) from a device queue, stage that instance's compiled
tables in shared memory, and their warps track the unit's paths. The launch is recorded once
in a CUDA graph and replayed.

    B = BatchTracker([total_degree_homotopy(F, g) for F, g in instances])
    results = B.solve()                   # list of Result, one per instance
    results = solve_batch(instances)      # the same in one call

Per n, two launch parameters can be chosen (``autotune`` measures them): the paths per work
unit, and in mixed precision the staging of the tables ("global": FP64 value coefficients
through L1/L2 and the rare FP64 areas in per-warp global slices, more warps per CTA; "shared":
everything in shared memory). Neither changes any result.
"""
from __future__ import annotations

import ctypes as ct
import time
from typing import Optional, Sequence

import numpy as np

from . import _lib
from .systems import TotalDegreeHomotopy, total_degree_homotopy, total_degree_start_solutions
from .tracking import (EndgameOptions, Result, TrackerOptions, _Handle, _path_results, make_options)


class InstanceDesc(ct.Structure):
    """hc_instance_desc (include/hcgpu.h)."""

    _fields_ = [("n", ct.c_int32), ("nG", ct.c_int32), ("nF", ct.c_int32), ("reserved", ct.c_int32),
                ("G_eq", ct.c_void_p), ("G_exps", ct.c_void_p), ("G_coef", ct.c_void_p),
                ("F_eq", ct.c_void_p), ("F_exps", ct.c_void_p), ("F_coef", ct.c_void_p),
                ("gamma_re", ct.c_double), ("gamma_im", ct.c_double), ("npaths", ct.c_int64)]


STAGING = {"global": 2, "shared": 1}


class BatchTracker:
    """Endgame trackers of many homotopies behind one handle and one launch."""

    def __init__(self, homotopies: Sequence[TotalDegreeHomotopy], tracker_options: Optional[TrackerOptions] = None,
                 endgame_options: Optional[EndgameOptions] = None, npaths: Optional[Sequence[int]] = None,
                 unit_paths: Optional[dict] = None, staging: Optional[dict] = None):
        self.tracker_options = tracker_options or TrackerOptions()
        self.options = endgame_options or EndgameOptions()
        self._h = _Handle(make_options(self.tracker_options, self.options))
        self._h.setup_step_control(self.tracker_options)
        self.unit_paths = dict(unit_paths or {})
        self.staging = dict(staging or {})
        self.set_homotopies(homotopies, npaths)

    def set_homotopies(self, homotopies: Sequence[TotalDegreeHomotopy], npaths: Optional[Sequence[int]] = None):
        """Replace the batch (hc_set_batch again) on the same handle: options, step model and
        device buffers are kept (monodromy's edges, parameter targets)."""
        self.homotopies = list(homotopies)
        if npaths is None:
            npaths = [int(np.prod(H.degrees)) for H in self.homotopies]
        self.npaths = np.asarray(npaths, dtype=np.int64)
        self.n = np.array([H.n for H in self.homotopies], dtype=np.int64)
        self.path_off = np.concatenate([[0], np.cumsum(self.npaths)])
        self.vec_off = np.concatenate([[0], np.cumsum(self.npaths * self.n)])
        self._upload()

    def _upload(self):
        descs = (InstanceDesc * len(self.homotopies))()
        keep = []
        for i, H in enumerate(self.homotopies):
            Ge, Gx, Gc = H.G.term_arrays()
            Fe, Fx, Fc = H.F.term_arrays()
            keep.append((Ge, Gx, Gc, Fe, Fx, Fc))
            d = descs[i]
            d.n, d.nG, d.nF = H.n, len(Ge), len(Fe)
            d.G_eq, d.G_exps, d.G_coef = Ge.ctypes.data, Gx.ctypes.data, Gc.ctypes.data
            d.F_eq, d.F_exps, d.F_coef = Fe.ctypes.data, Fx.ctypes.data, Fc.ctypes.data
            d.gamma_re, d.gamma_im = H.gamma.real, H.gamma.imag
            d.npaths = int(self.npaths[i])
        up = np.zeros(33, dtype=np.int32)
        for n, u in self.unit_paths.items():
            up[int(n)] = int(u)
        tp = np.zeros(1, dtype=np.int64)
        tv = np.zeros(1, dtype=np.int64)
        P = _lib.ptr
        rc = self._h.L.hc_set_batch(self._h.h, len(self.homotopies), descs, P(up), P(tp), P(tv))
        _lib.check(rc, self._h.h)
        assert int(tp[0]) == int(self.path_off[-1]) and int(tv[0]) == int(self.vec_off[-1])
        self.total_paths, self.total_elements = int(tp[0]), int(tv[0])
        self._plan()

    def _plan(self):
        up = np.zeros(33, dtype=np.int32)
        st = np.zeros(33, dtype=np.int32)
        for n, u in self.unit_paths.items():
            up[int(n)] = int(u)
        for n, v in self.staging.items():
            if v not in STAGING:
                raise ValueError(f"staging for n={n} must be one of {sorted(STAGING)}, got {v!r}")
            st[int(n)] = STAGING[v]
        P = _lib.ptr
        _lib.check(self._h.L.hc_set_batch_launch(self._h.h, P(up), P(st)), self._h.h)

    def set_unit_paths(self, unit_paths: dict):
        self.set_launch(unit_paths=unit_paths)

    def set_launch(self, unit_paths: Optional[dict] = None, staging: Optional[dict] = None):
        """Replace the per-n unit sizes and/or stagings (None keeps the current ones); the batch
        is re-planned without recompiling (hc_set_batch_launch)."""
        if unit_paths is not None:
            self.unit_paths = dict(unit_paths)
        if staging is not None:
            self.staging = dict(staging)
        self._plan()

    def autotune(self, starts=None, candidates=(2, 4, 8, 16, 32, 64), sample=60, repeats=1):
        """Measure and apply the fastest launch plan per n (hc_autotune_batch). Returns
        ({n: unit_paths}, {n: staging}, {(n, staging, unit_paths): ms per launch})."""
        if starts is None:
            starts = self.start_solutions()
        starts = np.ascontiguousarray(np.asarray(starts, dtype=np.complex128).reshape(-1))
        if starts.shape[0] != self.total_elements:
            raise ValueError(f"expected {self.total_elements} start values, got {starts.shape[0]}")
        cand = np.asarray(candidates, dtype=np.int32)
        up = np.zeros(33, dtype=np.int32)
        st = np.zeros(33, dtype=np.int32)
        ms = np.zeros(33 * 2 * len(cand), dtype=np.float64)
        P = _lib.ptr
        _lib.check(self._h.L.hc_autotune_batch(self._h.h, P(starts), int(sample or 0), P(cand), len(cand), repeats,
                                               P(up), P(st), P(ms)), self._h.h)
        mixed = self.tracker_options.precision == "mixed"
        names = {v: k for k, v in STAGING.items()}
        ns = sorted({int(n) for n in self.n})
        self.unit_paths = {n: int(up[n]) for n in ns}
        self.staging = {n: names.get(int(st[n]), "global") for n in ns} if mixed else {}
        table = {}
        ms = ms.reshape(33, 2, len(cand))
        for n in ns:
            for si, sname in enumerate(("global", "shared") if mixed else ("shared",)):
                for ci, c in enumerate(cand):
                    if np.isfinite(ms[n, si, ci]):
                        table[(n, sname, int(c))] = float(ms[n, si, ci])
        return dict(self.unit_paths), dict(self.staging), table

    def start_solutions(self):
        """Concatenated total-degree start solutions of every instance (src/total_degree.jl:240-262)."""
        out = np.empty(self.total_elements, dtype=np.complex128)
        for i, H in enumerate(self.homotopies):
            S = total_degree_start_solutions(H.degrees, np.arange(self.npaths[i]))
            out[self.vec_off[i]:self.vec_off[i + 1]] = S.reshape(-1)
        return out

    def track_arrays(self, starts=None):
        """Raw results (RESULT_DTYPE, all instances) and concatenated endpoints."""
        if starts is None:
            starts = self.start_solutions()
        starts = np.ascontiguousarray(np.asarray(starts, dtype=np.complex128).reshape(-1))
        if starts.shape[0] != self.total_elements:
            raise ValueError(f"expected {self.total_elements} start values, got {starts.shape[0]}")
        res = np.zeros(self.total_paths, dtype=_lib.RESULT_DTYPE)
        sol = np.zeros(self.total_elements, dtype=np.complex128)
        P = _lib.ptr
        _lib.check(self._h.L.hc_track_batch(self._h.h, P(starts), 1, P(res), P(sol)), self._h.h)
        return res, sol

    def split(self, res, sol):
        """Per-instance (results, endpoints[npaths, n]) views."""
        return [(res[self.path_off[i]:self.path_off[i + 1]],
                 sol[self.vec_off[i]:self.vec_off[i + 1]].reshape(-1, int(self.n[i])))
                for i in range(len(self.homotopies))]

    def solve(self, starts=None, seed=None, start_system="total_degree"):
        """One Result per instance; ``starts`` as for track_arrays (default: total-degree)."""
        flat = self.start_solutions() if starts is None else np.asarray(starts, dtype=np.complex128).reshape(-1)
        res, sol = self.track_arrays(flat)
        out = []
        for i, (r, x) in enumerate(self.split(res, sol)):
            n = int(self.n[i])
            zv = np.zeros((r.shape[0], n))
            zl = np.zeros((r.shape[0], n), dtype=np.complex128)
            Si = flat[self.vec_off[i]:self.vec_off[i + 1]].reshape(-1, n)
            prs = _path_results(r, x, zv, zl, Si, self.options.endgame_start)
            out.append(Result(prs, seed=seed, start_system=start_system))
        return out

    def stats(self):
        return self._h.stats()

    def cancel(self):
        self._h.cancel()


def solve_batch(instances, tracker_options=None, endgame_options=None, unit_paths=None, staging=None):
    """Solve many independent square systems by total-degree homotopies in one launch.
    ``instances``: (System, γ) pairs (as returned by systems.uneven_instances)."""
    Hs = [total_degree_homotopy(F, g) for F, g in instances]
    return BatchTracker(Hs, tracker_options, endgame_options, unit_paths=unit_paths, staging=staging).solve()


def autotune(homotopies, tracker_options=None, candidates=(2, 4, 8, 16, 32, 64), sample=None, repeats=1,
             verbose=False):
    """Choose the launch plan of every n of a batch of homotopies with the library's autotuner
    (hc_autotune_batch: for each n, ``sample`` instances of that n — all when None — tracked with
    every candidate unit size and, in mixed precision, both stagings, timed with CUDA events at
    the full batch's launch shape). Returns ({n: unit_paths}, {n: staging}); the staging dict is
    empty in FP64."""
    B = BatchTracker(homotopies, tracker_options)
    unit, staging, table = B.autotune(candidates=candidates, sample=sample, repeats=repeats)
    if verbose:
        for n in sorted(unit):
            row = {f"{c}/{s}": round(t, 2) for (m, s, c), t in table.items() if m == n}
            print(f"autotune n={n}:", row, "ms ->", (unit[n], staging.get(n, "shared")), flush=True)
    return unit, staging


def autotune_unit_paths(homotopies, tracker_options=None, candidates=(2, 4, 8, 16, 32, 64), sample=None,
                        repeats=1, verbose=False):
    """The unit sizes ``autotune`` chooses. Returns {n: unit_paths}."""
    return autotune(homotopies, tracker_options, candidates, sample=sample, repeats=repeats, verbose=verbose)[0]
