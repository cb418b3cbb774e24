"""GPU tests of batched tracking (hc_set_batch / hc_track_batch): many independent
homotopies of uneven size in one launch.

Every path of a batch runs the same per-path code as a single-homotopy launch, so its result
must equal, bit for bit, the one hc_track returns for its instance alone — whatever the work
unit sizes and however often the recorded graph is replayed. Small instances are also checked
against the CPU oracle."""
import numpy as np
import pytest

import hcgpu as hc
from _parity import REL_TOL, counts, oracle_track, rel_err
from hcgpu import _lib

pytestmark = pytest.mark.gpu

FIELDS = ["return_code", "t_re", "accuracy", "residual", "cond", "winding_number", "singular", "accepted_steps",
          "rejected_steps", "steps_eg", "path_number"]


def _batch(count, seed, max_n=8):
    inst = [(F, g) for F, g in hc.uneven_instances(count, seed) if F.n <= max_n]
    return [hc.total_degree_homotopy(F, g) for F, g in inst]


def _same(ra, xa, rb, xb):
    for f in FIELDS:
        a, b = ra[f], rb[f]
        assert np.array_equal(a, b, equal_nan=np.issubdtype(a.dtype, np.floating)), f
    assert np.array_equal(xa, xb)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_single_launches(precision):
    Hs = _batch(24, seed=11, max_n=6)
    to = hc.TrackerOptions(precision=precision)
    B = hc.BatchTracker(Hs, to)
    res, sol = B.track_arrays()
    assert res.shape[0] == B.total_paths == sum(int(np.prod(H.degrees)) for H in Hs)
    for i, (r, x) in enumerate(B.split(res, sol)):
        T = hc.EndgameTracker(Hs[i], hc.TrackerOptions(precision=precision))
        S = hc.total_degree_start_solutions(Hs[i].degrees)
        r1, x1, _, _ = T.track_arrays(S)
        _same(r, x, r1, x1)
        assert list(r["path_number"]) == list(range(1, r.shape[0] + 1))
    assert B.stats()["paths"] == B.total_paths


def test_unit_size_and_graph_replay_do_not_change_results():
    Hs = _batch(30, seed=12, max_n=7)
    B = hc.BatchTracker(Hs, hc.TrackerOptions(precision="mixed"))
    S = B.start_solutions()
    r0, x0 = B.track_arrays(S)
    r1, x1 = B.track_arrays(S)  # replay of the recorded graph
    _same(r0, x0, r1, x1)
    for up in ({n: 1 for n in range(3, 9)}, {n: 7 for n in range(3, 9)}, {3: 200, 5: 3, 8: 1000}):
        B.set_unit_paths(up)
        r2, x2 = B.track_arrays(S)
        _same(r0, x0, r2, x2)


def test_staging_per_n_does_not_change_results():
    """Mixed precision, each n staged in shared memory or with its FP64 areas in global slices,
    in every combination tried: bit-identical to hc_track of each instance alone."""
    Hs = _batch(30, seed=15, max_n=8)
    ns = sorted({H.n for H in Hs})
    B = hc.BatchTracker(Hs, hc.TrackerOptions(precision="mixed"), staging={n: "shared" for n in ns})
    S = B.start_solutions()
    r0, x0 = B.track_arrays(S)
    for i, (r, x) in enumerate(B.split(r0, x0)):
        T = hc.EndgameTracker(Hs[i], hc.TrackerOptions(precision="mixed"))
        r1, x1, _, _ = T.track_arrays(hc.total_degree_start_solutions(Hs[i].degrees))
        _same(r, x, r1, x1)
    alternate = {n: ("global" if k % 2 else "shared") for k, n in enumerate(ns)}
    for st in ({n: "global" for n in ns}, alternate):
        B.set_launch(staging=st)
        r2, x2 = B.track_arrays(S)
        _same(r0, x0, r2, x2)
        B.set_launch(unit_paths={n: 3 for n in ns})
        r3, x3 = B.track_arrays(S)
        _same(r0, x0, r3, x3)
    with pytest.raises(ValueError):
        B.set_launch(staging={ns[0]: "registers"})


def test_autotune_picks_valid_launch_parameters():
    """hc_autotune_batch times every (unit size, staging) pair per n, applies the fastest, and
    the tuned batch returns the default plan's results bit for bit."""
    Hs = _batch(16, seed=16, max_n=5)
    ns = {H.n for H in Hs}
    B = hc.BatchTracker(Hs, hc.TrackerOptions(precision="mixed"))
    r0, x0 = B.track_arrays()
    unit, staging, table = B.autotune(candidates=(2, 8), sample=4, repeats=1)
    assert set(unit) == ns and set(staging) == ns
    assert set(unit.values()) <= {2, 8} and set(staging.values()) <= {"global", "shared"}
    assert set(table) == {(n, s, c) for n in ns for s in ("global", "shared") for c in (2, 8)}
    assert all(t > 0 for t in table.values())
    for n in ns:  # the chosen pair is the fastest measured one
        assert table[(n, staging[n], unit[n])] == min(t for (m, _, _), t in table.items() if m == n)
    r, x = B.track_arrays()
    _same(r0, x0, r, x)
    unit64, staging64 = hc.autotune(Hs, hc.TrackerOptions(precision="fp64"), candidates=(4,), sample=2)
    assert set(unit64.values()) == {4} and staging64 == {}


def test_batch_against_oracle_small_instances():
    """Instances with n ≤ 4: counts equal to the oracle's and nonsingular endpoints within 1e-10."""
    Hs = _batch(40, seed=13, max_n=4)[:12]
    B = hc.BatchTracker(Hs)
    res, sol = B.track_arrays()
    for i, (r, x) in enumerate(B.split(res, sol)):
        S = hc.total_degree_start_solutions(Hs[i].degrees)
        ro, xo, _, _ = oracle_track(Hs[i], S)
        assert counts(r) == counts(ro)
        both = (ro["return_code"] == 1) & (ro["singular"] == 0) & (r["return_code"] == 1) & (r["singular"] == 0)
        if both.any():
            assert rel_err(x[both], xo[both]).max() <= REL_TOL


def test_solve_batch_results():
    inst = [(F, g) for F, g in hc.uneven_instances(10, 14) if F.n <= 5]
    results = hc.solve_batch(inst)
    assert len(results) == len(inst)
    for (F, g), R in zip(inst, results):
        assert len(R) == int(np.prod(F.degrees()))
        R1 = hc.solve(F, gamma=g)
        assert hc.nnonsingular(R) == hc.nnonsingular(R1)
        assert hc.nat_infinity(R) == hc.nat_infinity(R1)


def test_batch_learned_step_control():
    """The batch path honours the learned step control (same per-path code)."""
    from hcgpu import learn

    Hs = _batch(12, seed=15, max_n=6)
    to = hc.TrackerOptions(precision="mixed", step_control="learned", step_model=learn.default_model())
    B = hc.BatchTracker(Hs, to)
    res, sol = B.track_arrays()
    for i, (r, x) in enumerate(B.split(res, sol)):
        T = hc.EndgameTracker(Hs[i], to)
        r1, x1, _, _ = T.track_arrays(hc.total_degree_start_solutions(Hs[i].degrees))
        _same(r, x, r1, x1)
    assert B.stats()["learned_proposals"] > 0


def test_batch_rejects_bad_input():
    H = _batch(4, seed=16)[0]
    with pytest.raises(_lib.HCError, match="npaths"):
        hc.BatchTracker([H], npaths=[-1])
    B = hc.BatchTracker([H])
    with pytest.raises(ValueError):
        B.track_arrays(np.zeros(3, dtype=np.complex128))


def test_jump_check_with_learned_steps():
    """Three instances of the 2,000-instance workload (seed 0) on which learned steps made a
    path jump onto another path (two equal endpoints): the host entry points re-track the
    coincident paths with plain steps, so every endpoint matches the plain FP64 tracker's."""
    from hcgpu import learn

    inst = hc.uneven_instances(2000, 0)
    Hs = [hc.total_degree_homotopy(*inst[i]) for i in (278, 639, 1057)]
    B64 = hc.BatchTracker(Hs, hc.TrackerOptions(precision="fp64"))
    r64, x64 = B64.track_arrays()
    for precision in ("fp64", "mixed"):
        to = hc.TrackerOptions(precision=precision, step_control="learned", step_model=learn.default_model())
        B = hc.BatchTracker(Hs, to)
        r, x = B.track_arrays()
        # which paths jump depends on rounding-level details of the build; those that do are
        # re-tracked, and none of the results below may show a jump
        assert B.stats()["paths_retracked"] >= 0
        assert (r["return_code"] == r64["return_code"]).all()
        for (ri, xi), (r0, x0) in zip(B.split(r, x), B64.split(r64, x64)):
            ok = (ri["return_code"] == 1) & (r0["return_code"] == 1)
            assert rel_err(xi[ok], x0[ok]).max() <= 1e-10
        # the single-homotopy host entry point applies the same check
        T = hc.EndgameTracker(Hs[1], to)
        rs, xs, _, _ = T.track_arrays(hc.total_degree_start_solutions(Hs[1].degrees))
        r0, x0 = B64.split(r64, x64)[1]
        assert rel_err(xs, x0).max() <= 1e-10


def test_jump_check_retracks_coincident_endpoints():
    """Duplicated start solutions end at the same point by construction: with learned steps the
    host entry point flags every such pair and re-tracks both paths with plain steps, and the
    results equal the plain FP64 tracker's."""
    from hcgpu import learn

    F, g = hc.dense_random_system(4, 2, seed=3)
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    S2 = np.concatenate([S, S[:3]])  # paths 16, 17, 18 repeat paths 0, 1, 2
    r64, x64, _, _ = hc.EndgameTracker(H, hc.TrackerOptions(precision="fp64")).track_arrays(S2)
    for precision in ("fp64", "mixed"):
        to = hc.TrackerOptions(precision=precision, step_control="learned", step_model=learn.default_model())
        T = hc.EndgameTracker(H, to)
        r, x, _, _ = T.track_arrays(S2)
        nonsing = ((r64["return_code"] == 1) & (r64["singular"] == 0))[:3].sum()
        assert T.stats()["paths_retracked"] >= 2 * nonsing > 0
        assert (r["return_code"] == r64["return_code"]).all()
        ok = (r["return_code"] == 1) & (r64["return_code"] == 1)
        assert rel_err(x[ok], x64[ok]).max() <= 1e-10
