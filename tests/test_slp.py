"""Systems given as straight-line programs (hc_set_slp): the program is turned into CUDA C and
compiled by NVRTC with the tracking kernel. The CPU oracle tracks the same system twice — from
its expanded term table (independent of the program) and through its own program interpreter —
and both must give the GPU's return code on every path and nonsingular endpoints within 1e-10
relative, in FP64 and mixed precision.
The structured systems are passed unexpanded (products of linear forms; determinants by
elimination, with divisions); one system exercises every supported op."""
import math
import time

import numpy as np
import pytest

import hcgpu as hc
from hcgpu import slp
from _parity import REL_TOL, counts, oracle_track, rel_err

pytestmark = pytest.mark.gpu


def _check(P, S, gamma, precision, step_control="plain"):
    P.scaling = [float(np.max(np.abs(c))) for c in S.coefficients]  # the reference's G (total_degree.jl:62)
    H_tab = hc.total_degree_homotopy(S, gamma)
    starts = hc.total_degree_start_solutions(H_tab.degrees)
    ro, xo, _, _ = oracle_track(H_tab, starts)
    T = hc.EndgameTracker(slp.slp_homotopy(P, gamma), hc.TrackerOptions(precision=precision, step_control=step_control))
    rg, xg, _, _ = T.track_arrays(starts)
    bad = np.nonzero(ro["return_code"] != rg["return_code"])[0]
    assert bad.size == 0, (bad[:8], ro["return_code"][bad[:8]], rg["return_code"][bad[:8]])
    assert np.array_equal(ro["singular"], rg["singular"])
    ok = (ro["return_code"] == 1) & (ro["singular"] == 0)
    assert ok.sum() > 0
    assert rel_err(xg[ok], xo[ok]).max() <= REL_TOL
    # and the oracle evaluating the same program (its interpreter), path by path
    import hco

    rp, xp, _, _ = hco.track_slp(P, gamma, starts)
    assert np.array_equal(rp["return_code"], rg["return_code"])
    assert rel_err(xg[ok], xp[ok]).max() <= REL_TOL
    return ro, rg, T


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_products_of_linear_forms_unexpanded(precision):
    P, S = slp.products_of_linear_forms(4, 3, seed=1)
    ro, rg, T = _check(P, S, np.exp(2j * np.pi * 0.17), precision)
    assert counts(rg) == counts(ro)
    assert T.stats()["paths"] == 81


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_determinants_by_elimination(precision):
    P, S = slp.determinantal(3, 3, seed=2)
    _check(P, S, np.exp(2j * np.pi * 0.41), precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_every_supported_op(precision):
    P, S = slp.disguised_ops(0)
    _check(P, S, np.exp(2j * np.pi * 0.29), precision)


def test_program_of_a_term_table_matches_the_table_kernel():
    F, g = hc.dense_random_system(5, 2, seed=4)
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    r1, x1, _, _ = hc.EndgameTracker(H).track_arrays(S)
    T = hc.EndgameTracker(slp.slp_homotopy(slp.from_system(F), g))
    r2, x2, _, _ = T.track_arrays(S)
    assert np.array_equal(r1["return_code"], r2["return_code"])
    ok = (r1["return_code"] == 1) & (r1["singular"] == 0)
    assert rel_err(x2[ok], x1[ok]).max() <= REL_TOL
    # learned step control on the program's kernel: same codes
    T2 = hc.EndgameTracker(slp.slp_homotopy(slp.from_system(F), g), hc.TrackerOptions(step_control="learned"))
    r3, x3, _, _ = T2.track_arrays(S)
    assert np.array_equal(r1["return_code"], r3["return_code"])
    assert rel_err(x3[ok], x1[ok]).max() <= REL_TOL


def test_compiled_program_is_cached():
    P, S = slp.products_of_linear_forms(3, 2, seed=7)
    g = np.exp(2j * np.pi * 0.61)
    hc.EndgameTracker(slp.slp_homotopy(P, g))  # compiles (or finds the cubin on disk)
    t = time.perf_counter()
    T = hc.EndgameTracker(slp.slp_homotopy(P, g))
    assert time.perf_counter() - t < 2.0
    r, x, _, _ = T.track_arrays(hc.total_degree_start_solutions(P.degrees))
    assert (r["return_code"] == 1).sum() > 0


@pytest.mark.parametrize("d", [2, 6])
def test_reference_kat_x_minus_10_power_unexpanded(d):
    """test/endgame_test.jl:47-52: every path of (x-10)^d ends with winding number d. The
    reference evaluates (x-10)^d as written (ModelKit's program: a subtraction and a power);
    expanded into a term table, the residual near x = 10 is rounding noise below |x-10| ≈ 0.04
    for d = 6 (binomial coefficients up to 10^6), and no endgame can resolve the root. As a
    straight-line program it passes, in both precisions, for several γ."""
    (x,) = slp.variables(1)
    # the start system's scaling the reference computes from the expanded support (total_degree.jl:62)
    scale = max(float(math.comb(d, k)) * 10.0 ** (d - k) for k in range(d + 1))
    P = slp.Program([(x - 10.0) ** d], degrees=[d], scaling=[scale])
    import hco

    for precision in ("fp64", "mixed"):
        for k in range(3):
            g = np.exp(2j * np.pi * (0.05 + k / 3))
            starts = hc.total_degree_start_solutions([d])
            T = hc.EndgameTracker(slp.slp_homotopy(P, g), hc.TrackerOptions(precision=precision))
            r, xs, _, _ = T.track_arrays(starts)
            assert list(r["winding_number"]) == [d] * d, (precision, k, list(r["winding_number"]))
            assert (r["return_code"] == 1).all() and (r["singular"] == 1).all()
            assert np.abs(xs[:, 0] - 10).max() < 1e-6
            # the oracle evaluating the same program: same codes and winding numbers
            ro, xo, _, _ = hco.track_slp(P, g, starts)
            assert np.array_equal(ro["return_code"], r["return_code"])
            assert np.array_equal(ro["winding_number"], r["winding_number"])
