"""Learned step proposal: step-log collection, GPU training and held-out evaluation.

The tracker's plain step rule (update_stepsize!, src/tracker.jl:541-588) is conservative by
design. With ``step_control="learned"`` a 12→64→64→2 network (BF16 weights, FP32
accumulation; csrc/hc_mlp.cu) reads 12 features of the step just accepted and enlarges the
plain proposal of the next step by a factor f ∈ [1, max_factor], never beyond 0.75 τ (τ the
Padé trust region). Newton's contraction test still judges every step; a rejected enlarged
step falls back to the plain proposal. The network models the probability that Newton accepts
a step enlarged by f,

    P(accept | φ, f) = σ(k(φ) (o1(φ) − log f)),   k = softplus(o2) + 0.05,

and the tracker applies log f = o1 − logit(confidence)/k, i.e. the largest factor accepted with
probability ≥ ``confidence``.

Pipeline (``python -m hcgpu.learn all`` from the package directory, on a GPU):
  1. collect: the tracker runs with ``step_control="explore"`` (plain proposal × a pseudo-random
     f ∈ [1, 6]) over ``TRAIN_PATHS`` random start solutions of each of the 500 seeded training
     systems (10 dense cubics in 10 variables, seeds 1000–1499); every accepted-step decision
     is logged with its features, tried log f and outcome;
  2. train: mean/std feature normalisation, Adam on the GPU (hc_mlp_grad, hc_mlp_adam), the
     last 50 training systems held out for validation loss;
  3. tune: the confidence is chosen on 5 training systems (not the held-out ones);
  4. evaluate: 50 held-out seeded systems (seeds 2000–2049), plain FP64 vs plain mixed vs
     learned mixed: steps, time, counts, endpoint agreement.
The model (``step_model.npz``) is stored beside this file; the evaluation report goes to
``--eval-out`` (default ``step_model_eval.json`` in the working directory).
"""
from __future__ import annotations

import argparse
import json
import os
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .systems import dense_random_system, total_degree_homotopy, total_degree_start_solutions
from .tracking import TrackerOptions, _Handle, make_options

NFEAT = 12
FEATURES = ["t", "log10 previous Δs", "log10 τ (trust region)", "log10 θ (Newton contraction)",
            "log10 local error (predictor)", "log10 ‖x‖", "log10 ω", "log10 plain Δs / τ",
            "accepted fraction of the last 8 steps", "Newton iterations / 4", "log10 μ", "log10 plain Δs"]
NI, NH, NO = 12, 64, 2
NPARAMS = NH * NI + NH + NH * NH + NH + NO * NH + NO
HERE = os.path.dirname(os.path.abspath(__file__))
MODEL_PATH = os.path.join(HERE, "step_model.npz")
EVAL_PATH = "step_model_eval.json"
TRAIN_SEEDS = tuple(range(1000, 1500))
VAL_SEEDS = TRAIN_SEEDS[-50:]
TUNE_SEEDS = TRAIN_SEEDS[:5]
EVAL_SEEDS = tuple(range(2000, 2050))
FAMILY = dict(n=10, degree=3)
TRAIN_PATHS = 64
# step-log record fields (include/hcgpu.h)
F_ACCEPTED, F_FEAT, F_LOGF, F_VALID = 8, 20, 32, 34


@dataclass
class StepModel:
    params: np.ndarray
    mean: np.ndarray
    std: np.ndarray
    confidence: float = 0.8
    max_factor: float = 6.0
    meta: dict = field(default_factory=dict)

    def save(self, path=MODEL_PATH):
        np.savez(path, params=np.asarray(self.params, np.float32), mean=np.asarray(self.mean, np.float32),
                 std=np.asarray(self.std, np.float32), confidence=self.confidence, max_factor=self.max_factor,
                 meta=json.dumps(self.meta))

    @classmethod
    def load(cls, path=MODEL_PATH):
        z = np.load(path, allow_pickle=False)
        m = cls(params=z["params"].astype(np.float32), mean=z["mean"].astype(np.float32),
                std=z["std"].astype(np.float32), confidence=float(z["confidence"]),
                max_factor=float(z["max_factor"]), meta=json.loads(str(z["meta"])))
        if m.params.shape != (NPARAMS,) or m.mean.shape != (NFEAT,) or m.std.shape != (NFEAT,):
            raise ValueError(f"{path}: not a step model of this network")
        return m


def default_model() -> StepModel:
    """The shipped model, trained by this module on the 500 training systems."""
    if not os.path.exists(MODEL_PATH):
        raise FileNotFoundError(f"{MODEL_PATH} is missing: run `python -m hcgpu.learn all` on a GPU")
    return StepModel.load(MODEL_PATH)


def family_system(seed):
    F, g = dense_random_system(FAMILY["n"], FAMILY["degree"], seed=seed)
    return total_degree_homotopy(F, g)


def sample_starts(H, count, seed):
    total = int(np.prod(H.degrees))
    rng = np.random.Generator(np.random.PCG64(seed + 7919))
    idx = np.sort(rng.choice(total, size=min(count, total), replace=False))
    return total_degree_start_solutions(H.degrees, idx)


# ------------------------------------------------------------------------------ collect
def collect(seeds=TRAIN_SEEDS, paths_per_system=TRAIN_PATHS, precision="mixed", records_per_path=800,
            verbose=True):
    """Step logs of exploratory runs: features X, tried log-multipliers L, outcomes Y and the
    seed of the system of every record."""
    h = _Handle(make_options(TrackerOptions(precision=precision, step_control="explore")))
    cap = paths_per_system * records_per_path
    Xs, Ls, Ys, Ss = [], [], [], []
    t0 = time.time()
    for i, s in enumerate(seeds):
        H = family_system(s)
        S = sample_starts(H, paths_per_system, s)
        h.set_homotopy(H)
        h.set_step_log(cap, 0, S.shape[0])
        h.track(S)
        log = h.get_step_log(cap)
        log = log[log[:, F_VALID] == 1.0]
        Xs.append(log[:, F_FEAT:F_FEAT + NFEAT].astype(np.float32))
        Ls.append(log[:, F_LOGF].astype(np.float32))
        Ys.append(log[:, F_ACCEPTED].astype(np.float32))
        Ss.append(np.full(log.shape[0], s, dtype=np.int32))
        if verbose and (i + 1) % 50 == 0:
            print(f"collect: {i + 1}/{len(seeds)} systems, {sum(map(len, Ys))} records, {time.time() - t0:.1f} s",
                  flush=True)
    h.set_step_log(0)
    return dict(X=np.concatenate(Xs), L=np.concatenate(Ls), Y=np.concatenate(Ys), system=np.concatenate(Ss))


# ------------------------------------------------------------------------------ train
def init_params(seed=0):
    """He-uniform weights, zero biases."""
    rng = np.random.Generator(np.random.PCG64(seed))
    parts = []
    for fan_in, fan_out in ((NI, NH), (NH, NH), (NH, NO)):
        lim = np.sqrt(6.0 / fan_in)
        parts += [rng.uniform(-lim, lim, size=fan_out * fan_in), np.zeros(fan_out)]
    return np.concatenate(parts).astype(np.float32)


class _Trainer:
    """GPU training with the network kernels; torch supplies device memory and the stream."""

    def __init__(self, params):
        import torch

        self.torch = torch
        self.L = _lib.load()
        self.dev = torch.device("cuda")
        self.P = torch.from_numpy(np.asarray(params, np.float32)).to(self.dev)
        self.M = torch.zeros_like(self.P)
        self.V = torch.zeros_like(self.P)
        self.G = torch.zeros_like(self.P)
        self.loss = torch.zeros(1, device=self.dev)
        self.step = 0

    def stream(self):
        return ct_void(self.torch.cuda.current_stream().cuda_stream)

    def upload(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(self.dev)

    def grad(self, X, Lr, Y):
        rc = self.L.hc_mlp_grad(X.data_ptr(), Lr.data_ptr(), Y.data_ptr(), int(X.shape[0]), self.P.data_ptr(),
                                self.G.data_ptr(), self.loss.data_ptr(), self.stream())
        _lib.check(rc)

    def adam(self, lr, wd):
        self.step += 1
        _lib.check(self.L.hc_mlp_adam(self.P.data_ptr(), self.M.data_ptr(), self.V.data_ptr(), self.G.data_ptr(),
                                      self.step, float(lr), float(wd), self.stream()))

    def eval_loss(self, X, Lr, Y):
        self.grad(X, Lr, Y)
        return float(self.loss.item())

    def params(self):
        return self.P.cpu().numpy().copy()


def ct_void(v):
    import ctypes as ct

    return ct.c_void_p(int(v))


def train(data, steps=4000, batch=32768, lr=2e-3, weight_decay=1e-5, seed=0, verbose=True):
    X, Lr, Y, sysid = data["X"], data["L"], data["Y"], data["system"]
    val = np.isin(sysid, np.asarray(VAL_SEEDS))
    tr = ~val
    mean = X[tr].astype(np.float64).mean(0)
    std = np.maximum(X[tr].astype(np.float64).std(0), 1e-3)
    Xn = ((X - mean) / std).astype(np.float32)
    T = _Trainer(init_params(seed))
    Xv, Lv, Yv = T.upload(Xn[val]), T.upload(Lr[val]), T.upload(Y[val])
    ntr = int(tr.sum())
    Xt_h, Lt_h, Yt_h = Xn[tr], Lr[tr], Y[tr]
    rng = np.random.Generator(np.random.PCG64(seed))
    batch = min(batch, ntr)
    per_epoch = max(ntr // batch, 1)
    curve = []
    t0 = time.time()
    for it in range(steps):
        if it % per_epoch == 0:
            perm = rng.permutation(ntr)
            Xt, Lt, Yt = T.upload(Xt_h[perm]), T.upload(Lt_h[perm]), T.upload(Yt_h[perm])
        j = (it % per_epoch) * batch
        # cosine schedule with 100 warm-up steps
        w = min(1.0, (it + 1) / 100)
        cur = lr * w * (0.05 + 0.95 * 0.5 * (1 + np.cos(np.pi * it / steps)))
        T.grad(Xt[j:j + batch], Lt[j:j + batch], Yt[j:j + batch])
        T.adam(cur, weight_decay)
        if (it + 1) % 500 == 0 or it == steps - 1:
            tl = float(T.loss.item())
            vl = T.eval_loss(Xv, Lv, Yv) if Xv.shape[0] else float("nan")
            curve.append(dict(step=it + 1, train_loss=tl, val_loss=vl))
            if verbose:
                print(f"train: step {it + 1}/{steps} loss {tl:.4f} val {vl:.4f} ({time.time() - t0:.1f} s)", flush=True)
    # base rate: loss of the best constant predictor, for reference
    p = float(Y[val].mean()) if val.any() else float(Y.mean())
    base = -(p * np.log(p) + (1 - p) * np.log(1 - p)) if 0 < p < 1 else 0.0
    meta = dict(records=int(X.shape[0]), train_records=ntr, val_records=int(val.sum()), steps=steps, batch=batch,
                lr=lr, weight_decay=weight_decay, curve=curve, val_constant_loss=base,
                train_seeds=[TRAIN_SEEDS[0], TRAIN_SEEDS[-1]], val_seeds=[VAL_SEEDS[0], VAL_SEEDS[-1]],
                features=FEATURES, train_seconds=time.time() - t0)
    return StepModel(params=T.params(), mean=mean.astype(np.float32), std=std.astype(np.float32), meta=meta)


# ------------------------------------------------------------------------------ evaluate
def _run(h, S):
    import torch

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res, sol, val, last = h.track(S)
    dt = time.perf_counter() - t0
    st = h.stats()
    return res, sol, dt, st


def _counts(res):
    rc = res["return_code"]
    return dict(nonsingular=int(((rc == 1) & (res["singular"] == 0)).sum()),
                singular=int(((rc == 1) & (res["singular"] == 1)).sum()),
                at_infinity=int(((rc == 2) | (rc == 3)).sum()),
                failed=int((~np.isin(rc, [1, 2, 3, 14])).sum()))


def _endpoint_err(res_a, sol_a, res_b, sol_b):
    """max ‖x_a − x_b‖∞ / ‖x_b‖∞ over the paths nonsingular in both runs."""
    ok = (res_a["return_code"] == 1) & (res_a["singular"] == 0) & (res_b["return_code"] == 1) & \
        (res_b["singular"] == 0)
    if not ok.any():
        return 0.0
    den = np.abs(sol_b[ok]).max(axis=1)
    den = np.where(den == 0, 1.0, den)
    return float((np.abs(sol_a[ok] - sol_b[ok]).max(axis=1) / den).max())


def _baseline_modes():
    return {"fp64_plain": TrackerOptions(precision="fp64", step_control="plain"),
            "mixed_plain": TrackerOptions(precision="mixed", step_control="plain")}


def _run_modes(modes, seeds, paths_per_system):
    """Per seed and mode: (results, endpoints, seconds, stats)."""
    hs = {}
    for k, to in modes.items():
        hs[k] = _Handle(make_options(to))
        hs[k].setup_step_control(to)
    out = {}
    for s in seeds:
        H = family_system(s)
        S = sample_starts(H, paths_per_system, s + 1_000_003)
        for k in modes:
            hs[k].set_homotopy(H)
            _run(hs[k], S[:64])  # first launch of this program
            out[s, k] = _run(hs[k], S)
    return out


def compare(model, seeds, paths_per_system=4096, verbose=True, baseline=None):
    """FP64 plain vs mixed plain vs mixed learned on the given systems."""
    if baseline is None:
        baseline = _run_modes(_baseline_modes(), seeds, paths_per_system)
    learned = _run_modes({"mixed_learned": TrackerOptions(precision="mixed", step_control="learned",
                                                          step_model=model)}, seeds, paths_per_system)
    runs = {**baseline, **learned}
    modes = ["fp64_plain", "mixed_plain", "mixed_learned"]
    tot = {k: dict(seconds=0.0, steps=0, rejected=0, paths=0, proposals=0, proposals_rejected=0) for k in modes}
    per = []
    mism_codes = mism_counts = 0
    max_err = 0.0
    for s in seeds:
        for k in modes:
            res, sol, dt, st = runs[s, k]
            t = tot[k]
            t["seconds"] += dt
            t["steps"] += int(res["accepted_steps"].sum() + res["rejected_steps"].sum())
            t["rejected"] += int(res["rejected_steps"].sum())
            t["paths"] += res.shape[0]
            t["proposals"] += int(st["learned_proposals"])
            t["proposals_rejected"] += int(st["learned_rejected"])
        r64, x64 = runs[s, "fp64_plain"][:2]
        rl, xl = runs[s, "mixed_learned"][:2]
        rm, xm = runs[s, "mixed_plain"][:2]
        c64, cl, cm = _counts(r64), _counts(rl), _counts(rm)
        e_l = _endpoint_err(rl, xl, r64, x64)
        e_m = _endpoint_err(rm, xm, r64, x64)
        mc = int((rl["return_code"] != r64["return_code"]).sum())
        mism_codes += mc
        mism_counts += int(c64 != cl)
        max_err = max(max_err, e_l)
        per.append(dict(seed=s, counts_fp64=c64, counts_mixed=cm, counts_learned=cl, code_mismatch=mc,
                        endpoint_rel_err_learned=e_l, endpoint_rel_err_mixed=e_m))
        if verbose:
            print(f"seed {s}: fp64 {c64} learned {cl} mismatched codes {mc} err {e_l:.2e}", flush=True)
    summary = dict(systems=len(seeds), paths_per_system=paths_per_system, totals=tot,
                   systems_with_count_mismatch=mism_counts, path_code_mismatches=mism_codes,
                   max_endpoint_rel_err_learned_vs_fp64=max_err)
    for k in modes:
        t = tot[k]
        t["paths_per_second"] = t["paths"] / t["seconds"] if t["seconds"] else None
        t["steps_per_path"] = t["steps"] / max(t["paths"], 1)
    summary["speedup_learned_vs_fp64_plain"] = tot["fp64_plain"]["seconds"] / tot["mixed_learned"]["seconds"]
    summary["speedup_learned_vs_mixed_plain"] = tot["mixed_plain"]["seconds"] / tot["mixed_learned"]["seconds"]
    summary["step_reduction_learned_vs_mixed_plain"] = 1 - tot["mixed_learned"]["steps"] / tot["mixed_plain"]["steps"]
    return summary, per


def constant_model(multiplier: float, like: StepModel) -> StepModel:
    """A network that proposes the same multiplier at every step: all weights zero, output
    biases such that log f = log(multiplier) (o2 large makes the acceptance model sharp). It
    runs through the learned path's code unchanged — cap at 0.75 τ, fallback to the plain
    proposal on rejection, cooldown — so it separates what the network predicts from what
    any constant enlargement with the same safety rules gives."""
    params = np.zeros(NPARAMS, dtype=np.float32)
    o2 = 100.0
    k = o2 + 0.05
    conf = like.confidence
    params[-2] = np.log(multiplier) + np.log(conf / (1 - conf)) / k
    params[-1] = o2
    return StepModel(params=params, mean=np.zeros(NFEAT, np.float32), std=np.ones(NFEAT, np.float32),
                     confidence=conf, max_factor=like.max_factor, meta={"constant_multiplier": multiplier})


def _duplicates(res, sol):
    ok = (res["return_code"] == 1) & (res["singular"] == 0)
    X = sol[ok]
    if X.shape[0] == 0:
        return 0
    key = np.round(X / np.maximum(np.abs(X).max(1, keepdims=True), 1e-300), 8)
    _, cnt = np.unique(key.view(np.complex128).reshape(len(X), -1), axis=0, return_counts=True)
    return int((cnt > 1).sum())


def ablation(model, seeds=EVAL_SEEDS[:10], paths_per_system=4096, multipliers=(1.5, 2.0, 3.0), verbose=True):
    """Held-out systems, mixed precision: the reference's step rule with its default and FAST
    parameters (src/tracker.jl:58-62), the learned proposal, and constant multipliers with the
    learned path's cap and fallback; codes against the FP64 plain tracker, steps, time, and
    nonsingular endpoints found twice (path jumps within the sample). Device entry point
    (hc_track without the host's jump check is not used: the host call applies it to learned
    and constant runs alike)."""
    modes = {"fp64_plain": TrackerOptions(precision="fp64"),
             "mixed_plain": TrackerOptions(precision="mixed"),
             "mixed_fast": TrackerOptions(precision="mixed", parameters="fast"),
             "mixed_learned": TrackerOptions(precision="mixed", step_control="learned", step_model=model)}
    for m in multipliers:
        modes[f"mixed_const_{m:g}"] = TrackerOptions(precision="mixed", step_control="learned",
                                                      step_model=constant_model(m, model))
    runs = _run_modes(modes, seeds, paths_per_system)
    out = {}
    for k in modes:
        secs = steps = paths = mism = dup = retracked = 0
        cmis = 0
        for s in seeds:
            res, sol, dt, st = runs[s, k]
            r64 = runs[s, "fp64_plain"][0]
            secs += dt
            steps += int(res["accepted_steps"].sum() + res["rejected_steps"].sum())
            paths += res.shape[0]
            mism += int((res["return_code"] != r64["return_code"]).sum())
            cmis += int(_counts(res) != _counts(r64))
            dup += _duplicates(res, sol)
            retracked += int(st.get("paths_retracked", 0))
        out[k] = dict(paths_per_second=paths / secs, steps_per_path=steps / paths, code_mismatches_vs_fp64=mism,
                      systems_with_count_mismatch=cmis, duplicate_endpoints=dup, paths_retracked=retracked,
                      seconds=secs)
        if verbose:
            print(k, {a: round(b, 3) if isinstance(b, float) else b for a, b in out[k].items()}, flush=True)
    return dict(systems=list(seeds), paths_per_system=paths_per_system, modes=out)


def tune(model, confidences=(0.6, 0.7, 0.8, 0.9, 0.95), seeds=TUNE_SEEDS, paths_per_system=4096, verbose=True):
    """Pick the confidence with the fastest learned run whose counts and endpoints match FP64 on
    the tuning systems (training-family seeds, disjoint from the evaluation seeds)."""
    baseline = _run_modes(_baseline_modes(), seeds, paths_per_system)
    best, table = None, []
    for c in confidences:
        m = StepModel(params=model.params, mean=model.mean, std=model.std, confidence=c,
                      max_factor=model.max_factor, meta=model.meta)
        summ, _ = compare(m, seeds, paths_per_system, verbose=False, baseline=baseline)
        lt = summ["totals"]["mixed_learned"]
        row = dict(confidence=c, seconds=lt["seconds"], steps_per_path=lt["steps_per_path"],
                   mixed_plain_seconds=summ["totals"]["mixed_plain"]["seconds"],
                   count_mismatch=summ["systems_with_count_mismatch"], code_mismatch=summ["path_code_mismatches"],
                   err=summ["max_endpoint_rel_err_learned_vs_fp64"])
        table.append(row)
        if verbose:
            print("tune:", row, flush=True)
        if row["count_mismatch"] == 0 and row["err"] <= 1e-10 and (best is None or row["seconds"] < best["seconds"]):
            best = row
    if best is None:
        best = max(table, key=lambda r: r["confidence"])
    model.confidence = best["confidence"]
    model.meta["tuning"] = dict(seeds=list(seeds), paths_per_system=paths_per_system, table=table)
    return model


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("what", choices=["all", "evaluate", "ablation"])
    ap.add_argument("--train-paths", type=int, default=TRAIN_PATHS)
    ap.add_argument("--eval-paths", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--systems", type=int, default=len(TRAIN_SEEDS))
    ap.add_argument("--eval-systems", type=int, default=len(EVAL_SEEDS))
    ap.add_argument("--out", default=MODEL_PATH)
    ap.add_argument("--eval-out", default=EVAL_PATH)
    a = ap.parse_args(argv)
    if a.what == "all":
        data = collect(TRAIN_SEEDS[:a.systems], a.train_paths)
        print(f"collected {data['X'].shape[0]} records, acceptance {data['Y'].mean():.3f}", flush=True)
        model = train(data, steps=a.steps)
        model = tune(model)
        model.meta["train_paths_per_system"] = a.train_paths
        model.meta["systems"] = a.systems
        model.save(a.out)
        print("saved", a.out, flush=True)
    model = StepModel.load(a.out)
    if a.what == "ablation":
        out = ablation(model, EVAL_SEEDS[:a.eval_systems], a.eval_paths)
        with open(a.eval_out, "w") as f:
            json.dump(out, f, indent=1)
        return
    summ, per = compare(model, EVAL_SEEDS[:a.eval_systems], a.eval_paths)
    with open(a.eval_out, "w") as f:
        json.dump(dict(summary=summ, per_system=per, model=dict(confidence=model.confidence,
                                                                max_factor=model.max_factor)), f, indent=1)
    print(json.dumps(summ, indent=1))


if __name__ == "__main__":
    main()
