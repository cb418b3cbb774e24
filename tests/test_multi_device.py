"""Several library handles tracking contiguous ranges of one batch concurrently
(EndgameTracker(..., devices=[...])). The box has one GPU, so both handles sit on device 0:
the ranges, the concurrent calls and the gather are exercised, and every path's result must
equal, bit for bit, that of a single-handle call (per-path results do not depend on which
launch tracks the path)."""
import numpy as np
import pytest

import hcgpu as hc

pytestmark = pytest.mark.gpu

FIELDS = ["return_code", "t_re", "accuracy", "residual", "cond", "winding_number", "singular", "accepted_steps",
          "rejected_steps", "steps_eg", "path_number"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_two_handles_equal_one(precision):
    F, g = hc.dense_random_system(6, 2, seed=9)
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    to = hc.TrackerOptions(precision=precision)
    r1, x1, v1, l1 = hc.EndgameTracker(H, to).track_arrays(S)
    T2 = hc.EndgameTracker(H, hc.TrackerOptions(precision=precision), devices=[0, 0])
    r2, x2, v2, l2 = T2.track_arrays(S)
    for f in FIELDS:
        assert np.array_equal(r1[f], r2[f], equal_nan=r1[f].dtype.kind == "f"), f
    assert np.array_equal(x1, x2) and np.array_equal(l1, l2)
    assert list(r2["path_number"]) == list(range(1, len(S) + 1))
    assert T2.stats()["paths"] == len(S)
    R = hc.solve(F, gamma=g, precision=precision, devices=[0, 0])
    assert hc.nnonsingular(R) == int(((r1["return_code"] == 1) & (r1["singular"] == 0)).sum())
