"""Straight-line programs on the CPU: the tracer against expanded polynomials, the generated
CUDA C compiled by NVRTC for sm_103a (NVRTC needs no GPU), and the validation of programs at
the C ABI (hc_slp_source)."""
import ctypes as ct
import os

import numpy as np
import pytest

import hcgpu as hc
from hcgpu import _lib, slp

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "homotopycontinuation.jl_gb300", "csrc")
INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


@pytest.mark.parametrize("make", [lambda: slp.products_of_linear_forms(4, 3, 1), lambda: slp.determinantal(3, 3, 2),
                                  lambda: slp.disguised_ops(0), lambda: (slp.from_system(hc.dense_random_system(4, 2, seed=3)[0]),
                                                                         hc.dense_random_system(4, 2, seed=3)[0])])
def test_program_equals_its_expansion(make):
    P, S = make()
    rng = np.random.default_rng(5)
    for _ in range(5):
        x = rng.normal(size=P.n) + 1j * rng.normal(size=P.n)
        a, b = P.evaluate(x), S.evaluate(x)
        assert np.abs(a - b).max() <= 1e-13 * max(np.abs(b).max(), 1.0)
    assert list(P.degrees) == [int(d) for d in S.degrees()]


def _nvrtc():
    for path in ("/usr/local/cuda/lib64/libnvrtc.so", "libnvrtc.so"):
        try:
            return ct.CDLL(path)
        except OSError:
            continue
    pytest.skip("NVRTC not found")


def test_generated_source_compiles_with_nvrtc():
    P, _ = slp.disguised_ops(0)
    src = slp.source(P)
    assert "eval_vt" in src and "series3" in src and '#include "hc_track_kernel.cuh"' in src
    src += "template __global__ void hcd::track_kernel<true>(const __grid_constant__ hcd::Launch la);\n"
    L = _nvrtc()
    prog = ct.c_void_p()
    assert L.nvrtcCreateProgram(ct.byref(prog), src.encode(), b"slp.cu", 0, None, None) == 0
    opts = [b"--gpu-architecture=sm_103a", b"-std=c++17", b"-default-device", b"-diag-suppress=39,177",
            b"-I" + CSRC.encode(), b"-I" + INCLUDE.encode()]
    rc = L.nvrtcCompileProgram(prog, len(opts), (ct.c_char_p * len(opts))(*opts))
    n = ct.c_size_t()
    L.nvrtcGetProgramLogSize(prog, ct.byref(n))
    log = ct.create_string_buffer(n.value)
    L.nvrtcGetProgramLog(prog, log)
    assert rc == 0, log.value.decode()[:2000]
    L.nvrtcGetCUBINSize(prog, ct.byref(n))
    assert n.value > 100000
    L.nvrtcDestroyProgram(ct.byref(prog))


def _raw(instrs, nconst, consts, voff, tape, outs, n):
    ins = np.zeros(len(instrs), dtype=slp.INSTR_DTYPE)
    for k, (inp, op, out) in enumerate(instrs):
        ins[k]["input"] = list(inp) + [0] * (4 - len(inp))
        ins[k]["op"] = slp.OP[op]
        ins[k]["output"] = out
    c = np.asarray(consts, dtype=np.float64) if nconst else np.zeros(2)
    o = np.asarray(outs, dtype=np.int32)
    s = slp.hc_slp(n, len(ins), ins.ctypes.data, nconst, c.ctypes.data, voff, tape, o.ctypes.data)
    deg = np.full(n, 2, dtype=np.int32)
    sc = np.ones(n)
    L = _lib.load()
    ln = ct.c_int64()
    rc = L.hc_slp_source(ct.byref(s), _lib.ptr(deg), _lib.ptr(sc), None, 0, ct.byref(ln))
    return rc, L.hc_last_error(None).decode()


def test_program_validation():
    # slot 0 constant 1, slots 1..2 variables x, y; F = (x*y - 1, x + y)
    ok = [((1, 2), "MUL", 3), ((3, 0), "SUB", 4), ((1, 2), "ADD", 5)]
    assert _raw(ok, 1, [1.0, 0.0], 1, 6, [4, 5], 2)[0] == 0
    rc, msg = _raw([((1,), "EXP", 3)] + ok[1:], 1, [1.0, 0.0], 1, 6, [3, 5], 2)
    assert rc == 5 and "not supported" in msg  # HC_ERR_UNSUPPORTED
    rc, msg = _raw([((1, 4), "MUL", 3)] + ok[1:], 1, [1.0, 0.0], 1, 6, [4, 5], 2)
    assert rc == 1 and "not written before" in msg
    # a temporary slot may be written again (compacted tapes); a variable may not
    assert _raw(ok[:2] + [((1, 2), "ADD", 3)], 1, [1.0, 0.0], 1, 6, [4, 3], 2)[0] == 0
    rc, msg = _raw(ok[:2] + [((1, 2), "ADD", 2)], 1, [1.0, 0.0], 1, 6, [4, 5], 2)
    assert rc == 1 and "a constant, variable or parameter" in msg
    rc, msg = _raw(ok, 1, [1.0, 0.0], 1, 6, [4, 7], 2)
    assert rc == 1 and "never written" in msg
    rc, msg = _raw([((1, 99), "POW_INT", 3)] + ok[1:], 1, [1.0, 0.0], 1, 6, [4, 5], 2)
    assert rc == 5 and "exponent" in msg
