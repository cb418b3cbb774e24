"""Stopping a running tracking call from the host: hc_cancel from another thread (solve's
catch_interrupt, src/solve.jl:603-709) and the per-handle run time limit (HC_ERR_TIMEOUT).

Both stop the kernel between steps through a flag in mapped host memory; nothing here faults
or hangs a GPU. Paths finished before the stop keep exactly the results of an uninterrupted
call; the others report terminated_unknown."""
import ctypes as ct
import threading
import time

import numpy as np
import pytest

import hcgpu as hc
from hcgpu import _lib

pytestmark = pytest.mark.gpu

TERMINATED_UNKNOWN = hc.ENDGAME_CODES.index("terminated_unknown")


def _setup():
    F, g = hc.dense_random_system(10, 3, seed=0)  # 59,049 paths: several seconds in FP64
    H = hc.total_degree_homotopy(F, g)
    S = np.ascontiguousarray(hc.total_degree_start_solutions(H.degrees))
    T = hc.EndgameTracker(H, hc.TrackerOptions(precision="fp64"))
    return H, S, T


def _raw_track(T, S):
    h = T._h
    npaths = S.shape[0]
    res = np.zeros(npaths, dtype=_lib.RESULT_DTYPE)
    sol = np.zeros_like(S)
    P = _lib.ptr
    rc = h.L.hc_track(h.h, npaths, P(S), 1, 1.0, 0.0, 0.0, 0.0, P(res), P(sol), None, None)
    return rc, res, sol


def _check_partial(res, sol, ref_res, ref_sol):
    """Some paths stopped, some finished; the finished ones among the first len(ref_res) equal
    the uninterrupted call's results bit for bit."""
    done = res["return_code"] != TERMINATED_UNKNOWN
    assert 0 < done.sum() < len(res)
    m = len(ref_res)
    d = done[:m]
    for f in ("return_code", "accepted_steps", "rejected_steps", "singular", "winding_number", "accuracy"):
        assert np.array_equal(res[f][:m][d], ref_res[f][d], equal_nan=res[f].dtype.kind == "f"), f
    assert np.array_equal(sol[:m][d], ref_sol[d])
    assert np.array_equal(res["path_number"], np.arange(1, len(res) + 1))


def test_cancel_from_another_thread_and_time_limit():
    H, S, T = _setup()
    sub = S[:8192]
    rc, ref_res, ref_sol = _raw_track(T, sub)  # uninterrupted reference call
    assert rc == 0
    # hc_cancel from another thread while hc_track blocks (ctypes releases the GIL)
    timer = threading.Timer(0.2, T.cancel)
    t0 = time.perf_counter()
    timer.start()
    rc, res, sol = _raw_track(T, S)
    dt = time.perf_counter() - t0
    timer.join()
    assert rc == 4, _lib.load().hc_last_error(T._h.h)  # HC_ERR_CANCELLED
    assert dt < 3.0
    _check_partial(res, sol, ref_res, ref_sol)
    # the next call starts clean
    rc, res2, sol2 = _raw_track(T, sub)
    assert rc == 0 and np.array_equal(res2["return_code"], ref_res["return_code"])
    # time limit: the call stops itself
    T.set_time_limit(0.2)
    t0 = time.perf_counter()
    rc, res, sol = _raw_track(T, S)
    dt = time.perf_counter() - t0
    assert rc == 7, _lib.load().hc_last_error(T._h.h)  # HC_ERR_TIMEOUT
    assert dt < 3.0
    assert b"time limit" in _lib.load().hc_last_error(T._h.h)
    _check_partial(res, sol, ref_res, ref_sol)
    with pytest.raises(_lib.HCError) as e:
        T.track_arrays(S)
    assert e.value.code == 7
    T.set_time_limit(0)
    rc, res3, sol3 = _raw_track(T, sub)
    assert rc == 0 and np.array_equal(res3["return_code"], ref_res["return_code"])
    assert np.array_equal(sol3, ref_sol)


def test_time_limit_rejects_bad_values():
    _, _, T = _setup()
    with pytest.raises(_lib.HCError):
        T.set_time_limit(-1.0)
    with pytest.raises(_lib.HCError):
        T.set_time_limit(float("inf"))
