"""hc_track_noalloc: tracking without any device allocation by the library.

Callers that cannot call cudaMalloc (code under an allocator that owns all device memory, a
memory-capped sandbox, a hot path that must not allocate) use this entry point; its scratch
lives in a static device array of the library. The test compares it, through the C ABI and on
two calls in a row (the array keeps the previous call's contents), with the ordinary
hc_track entry point on the same homotopy and start solutions."""
import ctypes as ct

import numpy as np
import pytest

import hcgpu as hc
from hcgpu import _lib
from _parity import REL_TOL, rel_err

pytestmark = pytest.mark.gpu


def _noalloc(L, opts, H, d_starts, npaths, d_res, d_sol, stream):
    Ge, Gx, Gc = H.G.term_arrays()
    Fe, Fx, Fc = H.F.term_arrays()
    P = _lib.ptr
    return L.hc_track_noalloc(ct.byref(opts), H.n, len(Ge), P(Ge), P(Gx), P(Gc), len(Fe), P(Fe), P(Fx), P(Fc),
                              H.gamma.real, H.gamma.imag, npaths, ct.c_void_p(d_starts.data_ptr()), 1,
                              1.0, 0.0, 0.0, 0.0, ct.c_void_p(d_res.data_ptr()), ct.c_void_p(d_sol.data_ptr()),
                              ct.c_void_p(stream.cuda_stream))


def test_noalloc_matches_hc_track_twice():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    for seed, deg in ((1, 2), (3, 3)):
        F, g = hc.dense_random_system(6 if deg == 2 else 4, deg, seed=seed)
        H = hc.total_degree_homotopy(F, g)
        S = hc.total_degree_start_solutions(H.degrees)
        npaths, n = S.shape
        ref_res, ref_sol, _, _ = hc.EndgameTracker(H).track_arrays(S)  # existing entry point
        opts = hc.make_options()
        d_starts = torch.from_numpy(np.ascontiguousarray(S).view(np.float64).reshape(-1)).to(dev)
        for call in range(2):
            d_res = torch.full((npaths * _lib.RESULT_DTYPE.itemsize,), 0xAB, dtype=torch.uint8, device=dev)
            d_sol = torch.full((npaths * n * 2,), float("nan"), dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            rc = _noalloc(L, opts, H, d_starts, npaths, d_res, d_sol, stream)
            assert rc == 0, L.hc_last_error(None)
            stream.synchronize()
            res = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)
            sol = d_sol.cpu().numpy().view(np.complex128).reshape(npaths, n)
            assert (res["return_code"] == ref_res["return_code"]).all(), call
            assert (res["path_number"] == np.arange(1, npaths + 1)).all()
            ok = ref_res["return_code"] == 1
            assert rel_err(sol[ok], ref_sol[ok]).max() <= REL_TOL, call


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
