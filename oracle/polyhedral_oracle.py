"""CPU oracle of the polyhedral tracker (test infrastructure only).

Restates ``track(PT::PolyhedralTracker, (cell, x∞))`` (src/polyhedral.jl:412-530) on the C++
oracle: the toric homotopy from t = 0 to 1 (hco_track_toric; split at t₀ = clamp(0.1^(10/w_max),
0.9, 1 − 1e-6) and restarted with the weights rescaled to a maximum of 10 when the cell's largest
weight w_max is ≥ 10), then the coefficient homotopy t·F(x; start) + (1 − t)·F(x; target) with
the endgame (hco_track, γ = 1). The cells, start solutions and weights come from the host code
under test (hcgpu.polyhedral_homotopy); only the tracking is the oracle's.
"""
from __future__ import annotations

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import hco  # noqa: E402

TRACKER_SUCCESS = 1


def _terms(system):
    return system.term_arrays()


def track_toric(tracker, starts, nthreads=0):
    """The toric stage: (TrackerCode per path, endpoints at t = 1, accepted, rejected steps)."""
    x = starts.x
    rows = starts.cell_of
    npaths = len(x)
    Fs = _terms(tracker.generic_start)
    smax = np.array([tracker.wmax[c][0] for c in rows])
    split = smax >= 10
    t_end = np.where(split, np.clip(0.1 ** (10.0 / np.where(split, smax, 1.0)), 0.9, 1 - 1e-6), 1.0)
    o1 = hco.default_options(max_initial_step_size=0.2)
    res, sol = hco.track_toric(Fs, tracker.W1, x, rows, np.zeros(npaths), t_end, np.full(npaths, 20.0),
                               np.full(npaths, 1e-12), options=o1, nthreads=nthreads)
    codes = res["return_code"].copy()
    acc, rej = res["accepted_steps"].copy(), res["rejected_steps"].copy()
    omega, mu = res["omega"].copy(), res["mu"].copy()
    idx = np.nonzero(split & (codes == TRACKER_SUCCESS))[0]
    if len(idx):
        o2 = hco.default_options(min_step_size=0.0)
        smin2 = np.array([tracker.wmax[c][1] for c in rows[idx]])
        r2, s2 = hco.track_toric(Fs, tracker.W2, sol[idx], rows[idx], t_end[idx] ** (1.0 / smin2), np.ones(len(idx)),
                                 omega[idx], mu[idx], options=o2, nthreads=nthreads)
        codes[idx] = r2["return_code"]
        sol[idx] = s2
        acc[idx] += r2["accepted_steps"]
        rej[idx] += r2["rejected_steps"]
    return codes, sol, acc, rej


def track(tracker, starts, nthreads=0):
    """(codes, endpoints, toric codes) for every start solution of ``starts``
    (hcgpu.polyhedral_homotopy.PolyhedralStartSolutions) with the data of ``tracker``
    (hcgpu.polyhedral_homotopy.PolyhedralTracker). codes are EndgameTrackerCode values, or −1 where
    the toric stage failed (polyhedral_failed)."""
    codes, sol, _, _ = track_toric(tracker, starts, nthreads)
    npaths = len(sol)
    ok = codes == TRACKER_SUCCESS
    out_codes = np.full(npaths, -1, dtype=np.int64)
    out_x = sol.copy()
    k = np.nonzero(ok)[0]
    if len(k):
        r, xs, _, _ = hco.track(_terms(tracker.generic_start), _terms(tracker.target), 1.0 + 0j, sol[k],
                                endgame=True, nthreads=nthreads)
        out_codes[k] = r["return_code"]
        out_x[k] = xs
    return out_codes, out_x, codes
