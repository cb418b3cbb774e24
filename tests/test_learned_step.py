"""GPU tests of the step-proposal network kernels (against the FP64 oracle in
oracle/mlp_oracle.py) and of the learned step control in the tracker."""
import ctypes as ct

import numpy as np
import pytest

import hcgpu as hc
import mlp_oracle as M
from _parity import REL_TOL, counts, rel_err
from hcgpu import _lib, learn

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def _stream():
    import torch

    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


def _data(seed, B):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(B, M.NI)).astype(np.float32)
    L = rng.uniform(0, np.log(6.0), size=B).astype(np.float32)
    Y = (rng.uniform(size=B) < 0.6).astype(np.float32)
    p = M.init_params(seed + 1)
    p[M.NH * M.NI:M.NH * M.NI + M.NH] = rng.normal(scale=0.1, size=M.NH)
    return X, L, Y, p.astype(np.float32)


@pytest.mark.parametrize("B", [1, 37, 1000])
def test_forward_matches_oracle(B):
    lib = _lib.load()
    X, _, _, p = _data(10 + B, B)
    dX, dp = _dev(X), _dev(p)
    out = _dev(np.zeros((B, 2)))
    _lib.check(lib.hc_mlp_forward(dX.data_ptr(), B, dp.data_ptr(), out.data_ptr(), _stream()))
    o = out.cpu().numpy().astype(np.float64)
    ref, _ = M.forward(p, X, bf16=True)
    scale = np.abs(ref).max()
    assert np.abs(o - ref).max() <= 1e-4 * scale


@pytest.mark.parametrize("B", [16, 333, 20000])
def test_gradient_matches_oracle(B):
    """Loss and every parameter block of the gradient from hc_mlp_grad agree with the FP64
    oracle that rounds the same tensor-core operands to BF16."""
    lib = _lib.load()
    X, L, Y, p = _data(20 + B, B)
    dX, dL, dY, dp = _dev(X), _dev(L), _dev(Y), _dev(p)
    g = _dev(np.zeros(M.NPARAMS))
    loss = _dev(np.zeros(1))
    _lib.check(lib.hc_mlp_grad(dX.data_ptr(), dL.data_ptr(), dY.data_ptr(), B, dp.data_ptr(), g.data_ptr(),
                               loss.data_ptr(), _stream()))
    lr, gr = M.loss_and_grad(p, X, L, Y, bf16=True)
    lg = float(loss.cpu().numpy()[0])
    gg = g.cpu().numpy().astype(np.float64)
    assert abs(lg - lr) <= 1e-4 * abs(lr)
    o = 0
    for name, shape in M.SHAPES:
        k = int(np.prod(shape))
        a, b = gg[o:o + k], gr[o:o + k]
        assert np.linalg.norm(a - b) <= 2e-3 * np.linalg.norm(b) + 1e-7, name
        o += k
    # and the BF16 gradient is a descent direction of the exact FP64 loss
    _, g64 = M.loss_and_grad(p, X, L, Y)
    assert gg @ g64 > 0.9 * np.linalg.norm(gg) * np.linalg.norm(g64)


def test_adam_matches_oracle():
    lib = _lib.load()
    rng = np.random.default_rng(3)
    p = rng.normal(size=M.NPARAMS).astype(np.float32)
    g = rng.normal(size=M.NPARAMS).astype(np.float32)
    dp, dm, dv, dg = _dev(p), _dev(np.zeros(M.NPARAMS)), _dev(np.zeros(M.NPARAMS)), _dev(g)
    pr, mr, vr = p.astype(np.float64), np.zeros(M.NPARAMS), np.zeros(M.NPARAMS)
    for step in (1, 2, 3):
        _lib.check(lib.hc_mlp_adam(dp.data_ptr(), dm.data_ptr(), dv.data_ptr(), dg.data_ptr(), step, 1e-3, 1e-4,
                                   _stream()))
        pr, mr, vr = M.adam_step(pr, mr, vr, g.astype(np.float64), step, 1e-3, 1e-4)
    np.testing.assert_allclose(dp.cpu().numpy(), pr, rtol=1e-5, atol=1e-6)


def test_training_reduces_loss():
    """A few hundred GPU Adam steps fit a synthetic acceptance rule y = [ℓ < 0.8 + 0.5 x0]."""
    rng = np.random.default_rng(5)
    B = 8192
    X = rng.normal(size=(B, M.NI)).astype(np.float32)
    L = rng.uniform(0, np.log(6.0), size=B).astype(np.float32)
    Y = (L < 0.8 + 0.5 * X[:, 0]).astype(np.float32)
    T = learn._Trainer(learn.init_params(0))
    dX, dL, dY = T.upload(X), T.upload(L), T.upload(Y)
    l0 = T.eval_loss(dX, dL, dY)
    for _ in range(300):
        T.grad(dX, dL, dY)
        T.adam(3e-3, 0.0)
    l1 = T.eval_loss(dX, dL, dY)
    assert l1 < 0.5 * l0


def _family(seed, npaths):
    H = learn.family_system(seed)
    return H, learn.sample_starts(H, npaths, seed + 1_000_003)


def test_explore_step_log_records_features():
    H, S = _family(1000, 32)
    h = hc.tracking._Handle(hc.make_options(hc.TrackerOptions(precision="mixed", step_control="explore")))
    h.set_homotopy(H)
    h.set_step_log(32 * 800, 0, 32)
    res, sol, _, _ = h.track(S)
    log = h.get_step_log()
    valid = log[log[:, 34] == 1.0]
    assert valid.shape[0] > 10 * 32
    assert np.isfinite(valid[:, 20:32]).all()
    assert (valid[:, 32] >= 0).all() and (valid[:, 32] <= np.log(6.0) + 1e-6).all()
    assert (valid[:, 32] > 0.1).mean() > 0.5  # most steps explored an enlarged size
    assert (log[:, 35] == 2.0).all()  # mode field
    assert set(np.unique(valid[:, 8])) <= {0.0, 1.0}
    assert 0.0 < valid[:, 8].mean() < 1.0  # both outcomes present


def test_learned_needs_a_model():
    h = hc.tracking._Handle(hc.make_options(hc.TrackerOptions(step_control="learned")))
    H, S = _family(1000, 4)
    h.set_homotopy(H)
    with pytest.raises(_lib.HCError, match="hc_set_step_model"):
        h.track(S)
    bad = learn.StepModel(params=learn.init_params(0), mean=np.zeros(12, np.float32),
                          std=np.ones(12, np.float32), confidence=1.5)
    with pytest.raises(_lib.HCError, match="confidence"):
        h.set_step_model(bad)


def test_learned_step_gain_held_out():
    """The shipped model on held-out systems of the training family (seeds 2000-2001, never
    seen in training or tuning): identical codes and counts to the plain FP64 tracker, every
    nonsingular endpoint within 1e-10 of it, and fewer steps than plain step control."""
    model = learn.default_model()
    for seed in (2000, 2001):
        H, S = _family(seed, 1024)
        out = {}
        for name, to in {"fp64": hc.TrackerOptions(precision="fp64"),
                         "mixed": hc.TrackerOptions(precision="mixed"),
                         "learned": hc.TrackerOptions(precision="mixed", step_control="learned",
                                                      step_model=model)}.items():
            T = hc.EndgameTracker(H, to)
            out[name] = T.track_arrays(S) + (T.stats(),)
        r64, x64 = out["fp64"][0], out["fp64"][1]
        rl, xl, stl = out["learned"][0], out["learned"][1], out["learned"][4]
        rm = out["mixed"][0]
        assert counts(rl) == counts(r64)
        assert (rl["return_code"] == r64["return_code"]).all()
        both = (rl["return_code"] == 1) & (rl["singular"] == 0) & (r64["return_code"] == 1) & (r64["singular"] == 0)
        assert rel_err(xl[both], x64[both]).max() <= REL_TOL
        steps_l = int(rl["accepted_steps"].sum() + rl["rejected_steps"].sum())
        steps_m = int(rm["accepted_steps"].sum() + rm["rejected_steps"].sum())
        assert stl["learned_proposals"] > 0
        assert steps_l <= 0.9 * steps_m, (steps_l, steps_m)


def test_tracker_inference_matches_oracle():
    """The multiplier the tracker applies after an accepted step (step-log field 32) equals the
    oracle network on the logged features (fields 20..31, BF16-rounded weights), capped at
    0.75 τ / Δs_plain as the tracker caps it."""
    model = learn.default_model()
    H, S = _family(2002, 64)
    to = hc.TrackerOptions(precision="mixed", step_control="learned", step_model=model)
    T = hc.EndgameTracker(H, to)
    T._h.set_step_log(64 * 400, 0, 64)
    T.track_arrays(S)
    log = T._h.get_step_log()
    rec = log[(log[:, 34] == 1.0) & (log[:, 32] > 0)]
    assert rec.shape[0] > 64 * 10
    phi = rec[:, 20:32]
    pb = M.to_bf16(model.params)
    # biases stay FP32 on the device; only weights are BF16
    P = M.unpack(model.params.astype(np.float64))
    Q = M.unpack(pb)
    for b in ("b1", "b2", "b3"):
        Q[b] = P[b]
    net = M.propose_logf(M.pack(Q), model.mean.astype(np.float64), model.std.astype(np.float64), phi,
                         model.confidence, model.max_factor)
    cap = np.maximum(0.0, np.log(0.75) - np.log(10.0) * phi[:, 7])
    expect = np.minimum(net, cap)
    # the step is also clamped at the end of its segment (not logged), which only shortens it
    assert (rec[:, 32] <= expect + 1e-3).all()
    ok = np.abs(rec[:, 32] - expect) <= 1e-3
    assert ok.mean() >= 0.97, (ok.mean(), rec[~ok][:5, 32], expect[~ok][:5])


def test_learned_against_fast_preset_and_constant_multiplier():
    """What the network adds, on a held-out system (seed 2003, 1,024 paths, mixed precision):
    the learned proposal takes fewer steps than the reference's FAST_TRACKER_PARAMETERS
    (β_τ 0.75, β_ω_p 2; src/tracker.jl:58-62) and than plain control, with the FP64 tracker's
    codes on every path. A constant 3× proposal through the same safety rules (cap 0.75 τ,
    fallback to the plain proposal on rejection) is reported beside it: on held-out systems it
    comes within 2% of the network's step count, so the gain comes mostly from the safe
    enlargement itself."""
    model = learn.default_model()
    H, S = _family(2003, 1024)
    runs = {}
    for name, to in {"fp64": hc.TrackerOptions(precision="fp64"),
                     "plain": hc.TrackerOptions(precision="mixed"),
                     "fast": hc.TrackerOptions(precision="mixed", parameters="fast"),
                     "learned": hc.TrackerOptions(precision="mixed", step_control="learned", step_model=model),
                     "const3": hc.TrackerOptions(precision="mixed", step_control="learned",
                                                 step_model=learn.constant_model(3.0, model))}.items():
        r, x, _, _ = hc.EndgameTracker(H, to).track_arrays(S)
        runs[name] = (r, int(r["accepted_steps"].sum() + r["rejected_steps"].sum()))
    r64 = runs["fp64"][0]
    for name in ("fast", "learned", "const3"):
        assert np.array_equal(runs[name][0]["return_code"], r64["return_code"]), name
    steps = {k: v[1] for k, v in runs.items()}
    assert steps["learned"] < steps["fast"] < steps["plain"], steps
    assert abs(steps["const3"] - steps["learned"]) <= 0.1 * steps["learned"], steps
