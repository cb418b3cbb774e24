"""hc_track_noalloc: tracking without any device allocation by the library.

Callers that cannot call cudaMalloc (code under an allocator that owns all device memory, a
memory-capped sandbox, a hot path that must not allocate) use this entry point; its scratch
lives in a static device array of the library. The tests compare it, through the C ABI and on
two calls in a row (the array keeps the previous call's contents), with the ordinary
hc_track entry point on the same homotopy, options and start solutions, in both precisions,
with and without the endgame; the second call must leave the device's free memory unchanged.
A call on a stream that is being captured is refused (the tables are copied from a temporary
host buffer)."""
import ctypes as ct

import numpy as np
import pytest

import hcgpu as hc
from hcgpu import _lib
from _parity import REL_TOL, rel_err

pytestmark = pytest.mark.gpu


def _noalloc(L, opts, H, d_starts, npaths, d_res, d_sol, stream, endgame=1, t0=0.0):
    Ge, Gx, Gc = H.G.term_arrays()
    Fe, Fx, Fc = H.F.term_arrays()
    P = _lib.ptr
    return L.hc_track_noalloc(ct.byref(opts), H.n, len(Ge), P(Ge), P(Gx), P(Gc), len(Fe), P(Fe), P(Fx), P(Fc),
                              H.gamma.real, H.gamma.imag, npaths, ct.c_void_p(d_starts.data_ptr()), endgame,
                              1.0, 0.0, t0, 0.0, ct.c_void_p(d_res.data_ptr()), ct.c_void_p(d_sol.data_ptr()),
                              ct.c_void_p(stream.cuda_stream))


@pytest.mark.parametrize("endgame", [1, 0])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_matches_hc_track_twice(precision, endgame):
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    t0 = 0.0 if endgame else 1e-6  # the plain tracker stops short of the singular endpoints
    for seed, deg in ((1, 2), (3, 3)):
        F, g = hc.dense_random_system(6 if deg == 2 else 4, deg, seed=seed)
        H = hc.total_degree_homotopy(F, g)
        S = hc.total_degree_start_solutions(H.degrees)
        npaths, n = S.shape
        to = hc.TrackerOptions(precision=precision)
        if endgame:
            ref_res, ref_sol, _, _ = hc.EndgameTracker(H, to).track_arrays(S)  # existing entry point
        else:
            ref_res, ref_sol, _, _ = hc.Tracker(H, to).track_arrays(S, t1=1.0, t0=t0)
        opts = hc.make_options(to)
        d_starts = torch.from_numpy(np.ascontiguousarray(S).view(np.float64).reshape(-1)).to(dev)
        for call in range(2):
            d_res = torch.full((npaths * _lib.RESULT_DTYPE.itemsize,), 0xAB, dtype=torch.uint8, device=dev)
            d_sol = torch.full((npaths * n * 2,), float("nan"), dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info(dev)[0]
            rc = _noalloc(L, opts, H, d_starts, npaths, d_res, d_sol, stream, endgame, t0)
            assert rc == 0, L.hc_last_error(None)
            stream.synchronize()
            free_after = torch.cuda.mem_get_info(dev)[0]
            if call == 1:
                # the first call may load the kernel's module; the second allocates nothing
                assert free_after == free_before
            res = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)
            sol = d_sol.cpu().numpy().view(np.complex128).reshape(npaths, n)
            assert (res["return_code"] == ref_res["return_code"]).all(), call
            assert (res["path_number"] == np.arange(1, npaths + 1)).all()
            ok = ref_res["return_code"] == 1
            assert rel_err(sol[ok], ref_sol[ok]).max() <= REL_TOL, call


def test_noalloc_refuses_capture_and_unknown_step_control():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dev = torch.device("cuda", 0)
    F, g = hc.dense_random_system(3, 2, seed=5)
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    npaths, n = S.shape
    opts = hc.make_options()
    d_starts = torch.from_numpy(np.ascontiguousarray(S).view(np.float64).reshape(-1)).to(dev)
    d_res = torch.zeros((npaths * _lib.RESULT_DTYPE.itemsize,), dtype=torch.uint8, device=dev)
    d_sol = torch.zeros((npaths * n * 2,), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    # a successful call first: the array's address is looked up outside any capture
    assert _noalloc(L, opts, H, d_starts, npaths, d_res, d_sol, stream) == 0, L.hc_last_error(None)
    stream.synchronize()
    graph = torch.cuda.CUDAGraph()
    x = torch.zeros(4, device=dev)
    with torch.cuda.stream(stream):
        graph.capture_begin()
        x.add_(1.0)
        rc = _noalloc(L, opts, H, d_starts, npaths, d_res, d_sol, stream)
        graph.capture_end()
    assert rc == 5  # HC_ERR_UNSUPPORTED
    assert b"captured" in L.hc_last_error(None)
    graph.replay()
    torch.cuda.synchronize()
    assert x.tolist() == [1.0] * 4
    opts.step_control = 7
    assert _noalloc(L, opts, H, d_starts, npaths, d_res, d_sol, stream) == 1  # HC_ERR_INVALID_ARG


def test_noalloc_rejects_oversized_homotopy():
    L = _lib.load()
    F, g = hc.dense_random_system(10, 5, seed=0)  # 3003 monomials per equation: tables > 1 MiB
    H = hc.total_degree_homotopy(F, g)
    opts = hc.make_options()
    Ge, Gx, Gc = H.G.term_arrays()
    Fe, Fx, Fc = H.F.term_arrays()
    P = _lib.ptr
    rc = L.hc_track_noalloc(ct.byref(opts), H.n, len(Ge), P(Ge), P(Gx), P(Gc), len(Fe), P(Fe), P(Fx), P(Fc),
                            H.gamma.real, H.gamma.imag, 1, ct.c_void_p(16), 1, 1.0, 0.0, 0.0, 0.0,
                            ct.c_void_p(16), ct.c_void_p(16), None)
    assert rc == 6  # HC_ERR_TOO_LARGE, before any device work
    assert b"static scratch" in L.hc_last_error(None)
