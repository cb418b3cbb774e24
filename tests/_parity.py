"""Shared helpers for the GPU-vs-oracle parity tests."""
from __future__ import annotations

import numpy as np

import hco
import hcgpu as hc

# Relative endpoint tolerance of the parity protocol: ‖x_gpu − x_oracle‖∞ / ‖x_oracle‖∞ ≤ 1e-10
REL_TOL = 1e-10


def oracle_track(H, starts, endgame=True, t1=1.0, t0=0.0, options=None):
    return hco.track(H.G.term_arrays(), H.F.term_arrays(), H.gamma, starts, endgame=endgame, t1=t1, t0=t0,
                     options=options)


def rel_err(a, b):
    den = np.abs(b).max(axis=1)
    den = np.where(den == 0, 1.0, den)
    return np.abs(a - b).max(axis=1) / den


def compare_endgame(H, starts, precision="fp64", tracker_options=None, endgame_options=None,
                    oracle_options=None, tol=REL_TOL):
    """Track with the oracle and the GPU; return (oracle results, gpu results, rel errors of
    the paths that are nonsingular in both)."""
    to = tracker_options or hc.TrackerOptions()
    to.precision = precision
    T = hc.EndgameTracker(H, to, endgame_options)
    ro, xo, vo, lo = oracle_track(H, starts, options=oracle_options)
    rg, xg, vg, lg = T.track_arrays(starts)
    both = (ro["return_code"] == 1) & (ro["singular"] == 0) & (rg["return_code"] == 1) & (rg["singular"] == 0)
    err = rel_err(xg[both], xo[both]) if both.any() else np.zeros(0)
    return (ro, xo, vo), (rg, xg, vg), err


def counts(res):
    rc = res["return_code"]
    return dict(
        nonsingular=int(((rc == 1) & (res["singular"] == 0)).sum()),
        singular=int(((rc == 1) & (res["singular"] == 1)).sum()),
        at_infinity=int(((rc == 2) | (rc == 3)).sum()),
        failed=int((~np.isin(rc, [1, 2, 3, 14])).sum()),
    )
