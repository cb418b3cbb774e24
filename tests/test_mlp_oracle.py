"""CPU checks of the step-proposal network oracle and of the host side of the learned step
control (no GPU calls)."""
import os

import numpy as np
import pytest

import mlp_oracle as M
from hcgpu import learn


def _batch(rng, B):
    X = rng.normal(size=(B, M.NI))
    L = rng.uniform(0.0, np.log(6.0), size=B)
    Y = (rng.uniform(size=B) < 0.6).astype(np.float64)
    return X, L, Y


def test_layout_matches_the_package():
    assert M.NPARAMS == learn.NPARAMS == 5122
    assert learn.init_params(0).shape == (M.NPARAMS,)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = M.init_params(1).astype(np.float64)
    p[M.NH * M.NI:M.NH * M.NI + M.NH] = rng.normal(scale=0.1, size=M.NH)  # nonzero b1
    X, L, Y = _batch(rng, 40)
    _, g = M.loss_and_grad(p, X, L, Y)
    idx = np.concatenate([rng.choice(M.NPARAMS, 60, replace=False), [M.NPARAMS - 1, M.NPARAMS - 2]])
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (M.loss_and_grad(p + e, X, L, Y)[0] - M.loss_and_grad(p - e, X, L, Y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 * max(1.0, abs(g[i])), i


def test_bf16_rounding():
    a = np.array([1.0, 1.0 + 2**-8, 1.0 + 2**-7, 1.0 + 3 * 2**-8, -2.5, 0.0, 3.0e38], dtype=np.float32)
    r = M.to_bf16(a)
    # ties go to even: 1 + 2^-8 → 1, 1 + 3·2^-8 → 1 + 2^-6
    np.testing.assert_array_equal(r[:6], [1.0, 1.0, 1.0 + 2**-7, 1.0 + 2**-6, -2.5, 0.0])
    assert abs(r[6] - 3.0e38) / 3.0e38 < 2**-8


def test_bf16_forward_close_to_fp64():
    rng = np.random.default_rng(2)
    p = M.init_params(3)
    X, _, _ = _batch(rng, 64)
    o64, _ = M.forward(p, X)
    o16, _ = M.forward(p, X, bf16=True)
    assert np.abs(o16 - o64).max() <= 0.05 * np.abs(o64).max()


def test_loss_is_bce_of_the_acceptance_model():
    rng = np.random.default_rng(4)
    p = M.init_params(5).astype(np.float64)
    X, L, Y = _batch(rng, 16)
    loss, _ = M.loss_and_grad(p, X, L, Y)
    O, _ = M.forward(p, X)
    k = np.log1p(np.exp(O[:, 1])) + 0.05
    pr = 1 / (1 + np.exp(-k * (O[:, 0] - L)))
    bce = -np.mean(Y * np.log(pr) + (1 - Y) * np.log(1 - pr))
    assert abs(loss - bce) < 1e-12


def test_adam_step_descends():
    rng = np.random.default_rng(6)
    p = M.init_params(7).astype(np.float64)
    X, L, Y = _batch(rng, 256)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    l0, _ = M.loss_and_grad(p, X, L, Y)
    for step in range(1, 41):
        _, g = M.loss_and_grad(p, X, L, Y)
        p, m, v = M.adam_step(p, m, v, g, step, 1e-2, 0.0)
    l1, _ = M.loss_and_grad(p, X, L, Y)
    assert l1 < l0


def test_propose_logf_bounds():
    rng = np.random.default_rng(8)
    p = M.init_params(9)
    phi = rng.normal(size=(100, M.NI))
    lf = M.propose_logf(p, np.zeros(M.NI), np.ones(M.NI), phi, 0.8, 6.0)
    assert (lf >= 0).all() and (lf <= np.log(6.0) + 1e-12).all()


def test_step_model_save_load(tmp_path):
    m = learn.StepModel(params=learn.init_params(1), mean=np.arange(12, dtype=np.float32),
                        std=np.ones(12, dtype=np.float32), confidence=0.7, max_factor=5.0, meta={"a": 1})
    path = os.path.join(tmp_path, "m.npz")
    m.save(path)
    r = learn.StepModel.load(path)
    np.testing.assert_array_equal(r.params, m.params)
    np.testing.assert_array_equal(r.mean, m.mean)
    assert (r.confidence, r.max_factor, r.meta) == (0.7, 5.0, {"a": 1})


def test_shipped_step_model():
    """The committed model has this network's shapes, finite values and a validation loss
    below that of the best constant predictor."""
    if not os.path.exists(learn.MODEL_PATH):
        pytest.fail("shipped step model missing: run `python -m hcgpu.learn all` on a GPU")
    m = learn.default_model()
    assert np.isfinite(m.params).all() and np.isfinite(m.mean).all() and (m.std > 0).all()
    assert 0 < m.confidence < 1 and m.max_factor >= 1
    curve = m.meta["curve"]
    assert curve[-1]["val_loss"] < m.meta["val_constant_loss"]
