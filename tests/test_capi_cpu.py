"""Host-side checks that need no GPU: the C ABI library loads and exports every symbol of
include/hcgpu.h, its structs match the header's layout, defaults mirror the reference, and
argument errors come back as status codes."""
import ctypes as ct
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import hcgpu as hc
from hcgpu import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hcgpu.h")


def header_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(hc_\w+)\(", txt, re.M)))


def test_library_exports_header_symbols():
    L = _lib.load()
    names = header_functions()
    assert len(names) >= 10
    for nm in names:
        assert hasattr(L, nm), nm
    assert set(_lib.EXPORTS) == set(names)


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "hcgpu.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu\\n\", sizeof(hc_options), sizeof(hc_path_result),"
        " offsetof(hc_options, precision), offsetof(hc_path_result, accepted_steps),"
        " offsetof(hc_path_result, last_t));return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    so, sr, op, oa, ol = map(int, subprocess.run([str(exe)], capture_output=True, text=True).stdout.split())
    assert so == ct.sizeof(_lib.Options)
    assert sr == _lib.RESULT_DTYPE.itemsize
    assert op == _lib.Options.precision.offset
    assert oa == _lib.RESULT_DTYPE.fields["accepted_steps"][1]
    assert ol == _lib.RESULT_DTYPE.fields["last_t"][1]


def test_instance_desc_layout_matches_header(tmp_path):
    from hcgpu.batch import InstanceDesc

    src = tmp_path / "inst.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "hcgpu.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu\\n\", sizeof(hc_instance_desc), offsetof(hc_instance_desc, G_eq),"
        " offsetof(hc_instance_desc, gamma_re), offsetof(hc_instance_desc, npaths));return 0;}\n")
    exe = tmp_path / "inst"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    size, og, ogr, onp = map(int, subprocess.run([str(exe)], capture_output=True, text=True).stdout.split())
    assert size == ct.sizeof(InstanceDesc)
    assert og == InstanceDesc.G_eq.offset
    assert ogr == InstanceDesc.gamma_re.offset
    assert onp == InstanceDesc.npaths.offset


def test_certificate_layout_matches_header(tmp_path):
    src = tmp_path / "cert.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "hcgpu.h"\n'
        "int main(void){printf(\"%zu %zu %zu\\n\", sizeof(hc_certificate), offsetof(hc_certificate, enclosure),"
        " offsetof(hc_certificate, precision));return 0;}\n")
    exe = tmp_path / "cert"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    size, oe, op = map(int, subprocess.run([str(exe)], capture_output=True, text=True).stdout.split())
    assert size == _lib.CERT_DTYPE.itemsize
    assert oe == _lib.CERT_DTYPE.fields["enclosure"][1]
    assert op == _lib.CERT_DTYPE.fields["precision"][1]


def test_default_options_mirror_reference():
    o = _lib.default_options()
    # src/tracker.jl:45-62, :105-140 and src/endgame_tracker.jl:47-72
    assert (o.a, o.beta_a, o.beta_omega_p, o.beta_tau, o.strict_beta_tau, o.min_newton_iters) == (0.125, 1.0, 3.0, 0.4, 0.3, 2)
    assert (o.max_steps, o.extended_precision, o.min_step_size, o.terminate_cond) == (10000, 1, 1e-48, 1e13)
    assert (o.endgame_start, o.max_endgame_steps, o.max_endgame_extended_steps) == (0.1, 2000, 400)
    assert (o.min_cond, o.min_cond_growth, o.min_coord_growth, o.max_winding_number) == (1e6, 1e4, 100.0, 6)
    assert (o.val_finite_tol, o.val_at_infinity_tol, o.sing_cond, o.sing_accuracy) == (0.05, 0.01, 1e14, 1e-12)
    assert (o.singular_min_accuracy, o.scaling_threshold, o.refine_steps) == (1e-6, -30.0, 3)
    opts = hc.make_options(hc.TrackerOptions(parameters="conservative"))
    assert (opts.beta_omega_p, opts.beta_tau, opts.strict_beta_tau) == (4.0, 0.25, 0.1875)


def test_argument_errors_are_status_codes():
    L = _lib.load()
    assert L.hc_create(None, None) == 1
    assert L.hc_track(None, 1, None, 1, 1.0, 0.0, 0.0, 0.0, None, None, None, None) == 1
    assert L.hc_set_step_log(None, 10, 0, 1) == 1
    assert L.hc_last_error(None)
    o = _lib.default_options()
    h = ct.c_void_p()
    rc = L.hc_create(ct.byref(o), ct.byref(h))
    if rc == 0:  # a GPU is present: exercise the argument checks of a live handle
        assert L.hc_track(h, 4, None, 1, 1.0, 0.0, 0.0, 0.0, None, None, None, None) == 3  # no system yet
        assert L.hc_set_homotopy(h, 0, 0, None, None, None, 0, None, None, None, 1.0, 0.0) == 5
        L.hc_destroy(h)
    else:
        assert rc == 2 and b"hc_create" in L.hc_last_error(None)
    assert L.hc_set_toric(None, 2, 1, None, None, None, 1, None) == 1
    assert L.hc_track_toric(None, 1, None, None, None, None, None, None, None, None) == 1


def test_mixed_cells_entry_point():
    """hc_mixed_cells is host code: cyclic-5's cells through the C ABI, the count reported
    with HC_ERR_TOO_LARGE when the output is too small, and bad arguments as status codes."""
    from hcgpu import polyhedral_homotopy as ph

    L = _lib.load()
    P = _lib.ptr
    sup = ph.support_coefficients(hc.cyclic(5))[0]
    n = 5
    nterms = np.array([len(S) for S in sup], dtype=np.int32)
    pts = np.ascontiguousarray(np.concatenate(sup), dtype=np.int32)
    rng = np.random.default_rng(1)
    lif = np.ascontiguousarray(rng.integers(0, 2 ** 16, size=int(nterms.sum())), dtype=np.int64)
    cnt = np.zeros(1, dtype=np.int64)
    idx = np.zeros((4, 2 * n), dtype=np.int32)
    rc = L.hc_mixed_cells(n, P(nterms), P(pts), P(lif), 4, P(idx), None, None, None, P(cnt))
    assert rc in (1, 6)  # too many cells for 4 slots, or (rarely) a non-generic lifting
    if rc == 6:
        k = int(cnt[0])
        assert k > 4
        idx = np.zeros((k, 2 * n), dtype=np.int32)
        vol = np.zeros(k, dtype=np.int64)
        assert L.hc_mixed_cells(n, P(nterms), P(pts), P(lif), k, P(idx), None, None, P(vol), P(cnt)) == 0
        assert int(vol.sum()) == 70
        assert (idx[:, 0::2] != idx[:, 1::2]).all()
    bad = np.zeros(n, dtype=np.int32)
    assert L.hc_mixed_cells(n, P(bad), P(pts), P(lif), 4, None, None, None, None, P(cnt)) == 1
    assert L.hc_mixed_cells(0, P(nterms), P(pts), P(lif), 4, None, None, None, None, P(cnt)) == 1


def test_start_solutions_order():
    # src/total_degree.jl:240-262: product order with the first index fastest
    S = hc.total_degree_start_solutions([2, 3])
    assert S.shape == (6, 2)
    np.testing.assert_allclose(S[:, 0], [1, -1, 1, -1, 1, -1], atol=1e-15)
    np.testing.assert_allclose(S[:, 1], np.repeat(np.exp(2j * np.pi * np.arange(3) / 3), 2), atol=1e-15)


def test_total_degree_homotopy_scaling():
    F, g = hc.dense_random_system(3, 2, seed=4)
    H = hc.total_degree_homotopy(F, g)
    assert H.degrees == [2, 2, 2] and H.bezout_number() == 8
    for i in range(3):
        assert np.isclose(H.scaling[i], np.abs(F.coefficients[i]).max())
        x = np.array([0.3, -0.2 + 0.1j, 1.1])
        assert np.isclose(H.G.evaluate(x)[i], H.scaling[i] * (x[i] ** 2 - 1))


def test_multiplicities_and_counts():
    # src/unique_points.jl:314-341 and src/result.jl:161-212
    mk = lambda code, sol, sing, k: hc.PathResult(code, np.array(sol, complex), 0.0, 1e-14, 1e-14, sing, 1.0, None,
                                                   False, k, None, (None, 0.0), None, 1.0, 1e-16, 10, 0, 0, False)
    prs = [mk("success", [1, 2], False, 1), mk("success", [3, 3], True, 2), mk("success", [3, 3 + 1e-12], True, 3),
           mk("at_infinity", [1e9, 0], False, 4), mk("terminated_max_steps", [0, 0], False, 5)]
    R = hc.Result(prs)
    assert hc.nnonsingular(R) == 1 and hc.nat_infinity(R) == 1 and hc.nfailed(R) == 1
    assert hc.nsingular(R) == 1 and hc.nsingular(R, counting_multiplicities=True) == 2
    assert prs[1].multiplicity == 2


def test_shard_ranges_cover_batch():
    from hcgpu.parallel import shard_range

    for npaths in [0, 1, 7, 59049]:
        for world in [1, 2, 3, 8]:
            r = [shard_range(npaths, k, world) for k in range(world)]
            assert r[0][0] == 0 and r[-1][1] == npaths
            assert all(r[k][1] == r[k + 1][0] for k in range(world - 1))
            assert max(h - l for l, h in r) - min(h - l for l, h in r) <= 1


def _placeholder_track(starts):
    """Stand-in for a device call (no GPU here): per-path records numbered 1.. within the
    range, a code and an endpoint that depend only on the start solution."""
    import numpy as np

    from hcgpu import _lib

    res = np.zeros(len(starts), dtype=_lib.RESULT_DTYPE)
    res["path_number"] = np.arange(1, len(starts) + 1)
    res["return_code"] = 1 + (np.abs(starts).sum(axis=1) * 1e3).astype(np.int64) % 3
    res["accepted_steps"] = (np.angle(starts[:, 0]) * 100).astype(np.int64)
    return res, starts ** 2 + 1


def _gloo_worker(rank, world, port, out):
    import numpy as np
    import torch
    import torch.distributed as dist

    from hcgpu.parallel import shard_range, sharded_track

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lo, hi = shard_range(1000, rank, world)
    ms = torch.tensor([10.0 + rank])
    dist.all_reduce(ms, op=dist.ReduceOp.MAX)
    cnt = torch.tensor([hi - lo])
    dist.all_reduce(cnt)
    rng = np.random.default_rng(3)
    starts = rng.normal(size=(1001, 4)) + 1j * rng.normal(size=(1001, 4))  # same on every rank
    res, sol = sharded_track(_placeholder_track, starts)
    out.put((rank, lo, hi, float(ms.item()), int(cnt.item()), res.tobytes(), sol.tobytes()))
    dist.destroy_process_group()


def test_two_rank_sharding_gloo():
    import multiprocessing as mp
    import socket

    import numpy as np

    from hcgpu import _lib

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_gloo_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(60)
    assert got[0][1:3] == (0, 500) and got[1][1:3] == (500, 1000)
    assert all(g[3] == 11.0 and g[4] == 1000 for g in got)
    # every rank holds the whole batch, equal to tracking it as one range
    rng = np.random.default_rng(3)
    starts = rng.normal(size=(1001, 4)) + 1j * rng.normal(size=(1001, 4))
    ref_res, ref_sol = _placeholder_track(starts)
    for g in got:
        res = np.frombuffer(g[5], dtype=_lib.RESULT_DTYPE)
        sol = np.frombuffer(g[6], dtype=np.complex128).reshape(-1, 4)
        assert np.array_equal(res, ref_res) and np.array_equal(sol, ref_sol)


def test_track_on_handles_gathers_in_path_order():
    """The one-process form over stand-in handles (no GPU): ranges, renumbering and order."""
    import numpy as np

    from hcgpu.parallel import merge_stats, track_on_handles

    class FakeHandle:
        n = 4

        def track(self, starts, endgame=True, t1=1.0, t0=0.0):
            r, x = _placeholder_track(starts)
            return r, x, np.abs(x), x.conj()

    rng = np.random.default_rng(4)
    starts = rng.normal(size=(37, 4)) + 1j * rng.normal(size=(37, 4))
    for k in (1, 2, 3, 5):
        res, sol, val, last = track_on_handles([FakeHandle() for _ in range(k)], starts)
        ref_res, ref_sol = _placeholder_track(starts)
        assert np.array_equal(res, ref_res) and np.array_equal(sol, ref_sol)
        assert np.array_equal(last, ref_sol.conj())
    st = merge_stats([{"paths": 3.0, "monomials": 7.0, "clk_run": 1.0}, {"paths": 4.0, "monomials": 7.0, "clk_run": 2.0}])
    assert st == {"paths": 7.0, "monomials": 7.0, "clk_run": 3.0}
