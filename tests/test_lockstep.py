"""Lockstep scheduling of a CTA's warps (hc_options::lockstep): every warp advances its path by
one step per round and the CTA (mode 1) or the warps sharing an SM sub-partition (mode 2) wait
for each other, so the warps run the same code together. Each path still runs the same
operations in the same order, so results must be identical bit for bit to the per-warp
schedule, for single launches and for batches, in both precisions; the automatic choice takes
mode 1 with 8 or more warps per CTA (mode 3 for large mixed-precision programs), and mode 1 for
batches."""
import numpy as np
import pytest

import hcgpu as hc

pytestmark = pytest.mark.gpu

FIELDS = ["return_code", "t_re", "accuracy", "residual", "cond", "winding_number", "singular", "accepted_steps",
          "rejected_steps", "steps_eg", "path_number"]


def _same(ra, xa, rb, xb):
    for f in FIELDS:
        a, b = ra[f], rb[f]
        assert np.array_equal(a, b, equal_nan=np.issubdtype(a.dtype, np.floating)), f
    assert np.array_equal(xa, xb)


@pytest.mark.parametrize("precision,step_control", [("mixed", "learned"), ("mixed", "plain"), ("fp64", "plain")])
def test_lockstep_equals_per_warp_schedule(precision, step_control):
    F, g = hc.dense_random_system(7, 3, seed=2)  # 2,187 paths; 8 warps per CTA fit in both layouts
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    out = {}
    for mode in (0, 1, 2, 3, -1):
        to = hc.TrackerOptions(precision=precision, step_control=step_control, warps_per_cta=8, lockstep=mode)
        T = hc.EndgameTracker(H, to)
        r, x, _, _ = T.track_arrays(S)
        out[mode] = (r, x, T.stats())
    for mode in (1, 2, 3, -1):
        _same(out[0][0], out[0][1], out[mode][0], out[mode][1])
    assert [out[m][2]["lockstep"] for m in (0, 1, 2, 3)] == [0, 1, 2, 3]
    assert out[-1][2]["lockstep"] == 1  # automatic with 8 warps per CTA and 854 value terms
    # the plain tracker (no endgame) through the same kernel
    r0, x0 = [], []
    for mode in (0, 1, 2, 3):
        T = hc.Tracker(H, hc.TrackerOptions(precision=precision, warps_per_cta=8, lockstep=mode))
        r, x, _, _ = T.track_arrays(S[:512], t1=1.0, t0=0.1)
        r0.append(r)
        x0.append(x)
    for m in (1, 2, 3):
        for f in ("return_code", "accepted_steps", "rejected_steps", "t_re"):
            assert np.array_equal(r0[0][f], r0[m][f]), f
        assert np.array_equal(x0[0], x0[m])


def test_automatic_schedule_and_warp_counts():
    """Up to 16 warps per CTA for single homotopies (bit-identical results); the automatic mode
    takes groups of two sub-partitions for large mixed-precision programs (≥ 2,000 value
    terms) and the CTA-wide barrier otherwise."""
    F, g = hc.dense_random_system(6, 3, seed=4)  # small tables: 16 warps fit
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    runs = {}
    for w in (8, 16):
        T = hc.EndgameTracker(H, hc.TrackerOptions(precision="mixed", warps_per_cta=w))
        r, x, _, _ = T.track_arrays(S)
        runs[w] = (r, x, T.stats())
    _same(runs[8][0], runs[8][1], runs[16][0], runs[16][1])
    assert runs[16][2]["warps_per_block"] == 16 and runs[16][2]["lockstep"] == 1
    T = hc.EndgameTracker(H, hc.TrackerOptions(precision="mixed"))
    T.track_arrays(S[:64])
    assert T.stats()["warps_per_block"] == 16  # as many as fit, at most 16
    F10, g10 = hc.dense_random_system(10, 3, seed=0)  # 2,880 value terms, 13 warps fit
    H10 = hc.total_degree_homotopy(F10, g10)
    S10 = hc.total_degree_start_solutions(H10.degrees)[:1024]
    T = hc.EndgameTracker(H10, hc.TrackerOptions(precision="mixed"))
    r, x, _, _ = T.track_arrays(S10)
    assert T.stats()["lockstep"] == 3 and T.stats()["warps_per_block"] == 13
    r0, x0, _, _ = hc.EndgameTracker(H10, hc.TrackerOptions(precision="mixed", lockstep=0)).track_arrays(S10)
    _same(r0, x0, r, x)
    with pytest.raises(hc._lib.HCError):
        hc.EndgameTracker(H, hc.TrackerOptions(warps_per_cta=17))


def test_lockstep_in_batches():
    inst = [(F, g) for F, g in hc.uneven_instances(40, 17) if F.n <= 7]
    Hs = [hc.total_degree_homotopy(F, g) for F, g in inst]
    res = []
    for mode in (0, 1, 2, 3):
        B = hc.BatchTracker(Hs, hc.TrackerOptions(precision="mixed", step_control="learned", lockstep=mode))
        r, x = B.track_arrays()
        res.append((r, x, B.stats()))
    for m in (1, 2, 3):
        _same(res[0][0], res[0][1], res[m][0], res[m][1])
    assert [r[2]["lockstep"] for r in res] == [0, 1, 2, 3]
    B = hc.BatchTracker(Hs, hc.TrackerOptions(precision="mixed", step_control="learned"))
    r, x = B.track_arrays()
    _same(res[0][0], res[0][1], r, x)
    assert B.stats()["lockstep"] == (1 if B.stats()["warps_per_block"] >= 8 else 0)
    # more than 8 warps per CTA (as many as fit, at most 16) against 8 and 4: the same results
    assert B.stats()["warps_per_block"] > 8
    for w in (8, 4):
        Bw = hc.BatchTracker(Hs, hc.TrackerOptions(precision="mixed", step_control="learned", warps_per_cta=w))
        rw, xw = Bw.track_arrays()
        assert Bw.stats()["warps_per_block"] == w
        _same(r, x, rw, xw)


def test_lockstep_option_is_validated():
    F, g = hc.dense_random_system(3, 2, seed=1)
    with pytest.raises(hc._lib.HCError):
        hc.EndgameTracker(hc.total_degree_homotopy(F, g), hc.TrackerOptions(lockstep=4))
