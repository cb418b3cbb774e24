"""CPU oracle of the step-proposal network (test infrastructure only).

Restates, in NumPy FP64, the 12→64→64→2 network, its loss and its gradient as the CUDA
kernels of homotopycontinuation.jl_gb300/csrc/hc_mlp.cu compute them. HomotopyContinuation.jl has
no learned step control (its step size comes from the closed-form rule of src/tracker.jl:541-588),
so there is no reference output to pin this oracle to: it is pinned instead by a central finite
difference check of its own analytic gradient (tests/test_mlp_oracle.py).

``bf16=True`` rounds every tensor-core operand to BF16 (round to nearest even) exactly where the
GPU kernels do — X, W1, H1, W2, H2, W3 in the forward pass; dH2, H1, W2, dH1, X in the backward
pass — so that the GPU results can be compared with a tolerance set by FP32 accumulation order
only. Only tests may import this module.

Parameter layout (FP32 vector, row-major): W1[64][12] b1[64] W2[64][64] b2[64] W3[2][64] b3[2].
Loss of one logged step with features x, tried log-multiplier ℓ and outcome y ∈ {0, 1}:
    k = softplus(o2) + 0.05,  z = k (o1 − ℓ),  L = softplus(z) − y z      (mean over the batch)
"""
from __future__ import annotations

import numpy as np

NI, NH, NO = 12, 64, 2
SHAPES = [("W1", (NH, NI)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NO, NH)), ("b3", (NO,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    out, o = {}, 0
    for name, shape in SHAPES:
        k = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + k], dtype=np.float64).reshape(shape)
        o += k
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SHAPES])


def to_bf16(a):
    """Round FP32 values to BF16 (nearest even) and return them as float64."""
    u = np.ascontiguousarray(np.asarray(a, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _r(a, bf16):
    return to_bf16(a) if bf16 else np.asarray(a, dtype=np.float64)


def softplus(x):
    return np.where(x > 20.0, x, np.log1p(np.exp(np.minimum(x, 20.0))))


def sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def init_params(seed: int = 0):
    """He-uniform weights, zero biases (the training script's initialisation)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = {}
    for name, shape in SHAPES:
        if name.startswith("W"):
            lim = np.sqrt(6.0 / shape[1])
            d[name] = rng.uniform(-lim, lim, size=shape)
        else:
            d[name] = np.zeros(shape)
    return pack(d).astype(np.float32)


def forward(p, X, bf16=False):
    """Returns (O[B,2], cache)."""
    P = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    A1 = _r(X, bf16) @ _r(P["W1"], bf16).T + P["b1"]
    H1 = np.maximum(A1, 0.0)
    if bf16:
        H1 = H1.astype(np.float32).astype(np.float64)  # stored FP32 in shared memory
    A2 = _r(H1, bf16) @ _r(P["W2"], bf16).T + P["b2"]
    H2 = np.maximum(A2, 0.0)
    if bf16:
        H2 = H2.astype(np.float32).astype(np.float64)
    O = _r(H2, bf16) @ _r(P["W3"], bf16).T + P["b3"]
    return O, (P, X, H1, H2)


def loss_and_grad(p, X, L, Y, bf16=False):
    """Mean loss and its gradient with respect to the parameter vector."""
    O, (P, X, H1, H2) = forward(p, X, bf16)
    B = X.shape[0]
    L = np.asarray(L, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    o1, o2 = O[:, 0], O[:, 1]
    k = softplus(o2) + 0.05
    z = k * (o1 - L)
    loss = float(np.mean(softplus(z) - Y * z))
    dz = (sigmoid(z) - Y) / B
    dO = np.stack([dz * k, dz * (o1 - L) * sigmoid(o2)], axis=1)
    g = {}
    g["W3"] = dO.T @ H2  # CUDA cores on the GPU: not rounded
    g["b3"] = dO.sum(0)
    dH2 = (dO @ P["W3"]) * (H2 > 0)
    g["b2"] = dH2.sum(0)
    g["W2"] = _r(dH2, bf16).T @ _r(H1, bf16)
    dH1 = (_r(dH2, bf16) @ _r(P["W2"], bf16)) * (H1 > 0)
    g["b1"] = dH1.sum(0)
    g["W1"] = _r(dH1, bf16).T @ _r(X, bf16)
    return loss, pack(g)


def adam_step(p, m, v, g, step, lr, weight_decay, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step with L2 weight decay added to the gradient (the GPU kernel's update)."""
    g = g + weight_decay * p
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def propose_logf(p, mean, std, phi, confidence, max_factor):
    """Log step multiplier the tracker applies: clamp(o1 − logit(confidence)/k, 0, log max_factor)."""
    x = (np.asarray(phi, dtype=np.float64) - mean) / std
    O, _ = forward(p, x[None, :] if x.ndim == 1 else x)
    k = softplus(O[:, 1]) + 0.05
    c = np.log(confidence / (1 - confidence))
    lf = O[:, 0] - c / k
    return np.clip(lf, 0.0, np.log(max_factor))
