"""Parameter homotopies on the GPU tracker.

The reference's ``ParameterHomotopy`` (src/homotopies/parameter_homotopy.jl:3-44) is

    H(x, t) = F(x; t p + (1 - t) q),   p = start_parameters, q = target_parameters.

When the parameters enter the coefficients affinely — c_k(p) = c0_k + Σ_j C_kj p_j, the
common case of coefficient-parameter homotopies — this equals

    H(x, t) = t F(x; p) + (1 - t) F(x; q),

which is the straight-line homotopy the GPU kernel tracks (γ t G + (1 - t) F with G = F(·; p),
F = F(·; q), γ = 1). Any other dependence on the parameters goes through a straight-line
program with parameters (``hcgpu.slp``): the parameters are inputs of the generated evaluator,
computed at each t as t p + (1 - t) q, with the series p(t + s) = p(t) + s (p - q) in the
predictor's Taylor coefficients — the reference's ParameterHomotopy itself.
``parametric_system(polys, nvars, nparams)`` picks the form: term tables when the parameters
enter affinely, a program otherwise.

API, mirroring the reference:

* ``parametric_system(polys, nvars, nparams)`` — ``System(eqs, variables, parameters)``;
  ``ParametricSystem.from_polys`` for the affine case; ``F(p)`` (``Program.fixed(p)``) fixes the
  parameters (``fix_parameters``, src/systems/fixed_parameter_system.jl).
* ``ParameterHomotopy(F, p, q)`` / ``parameter_homotopy(F; start_parameters, target_parameters)``
  (src/solve.jl:233-260), usable with ``Tracker`` and ``EndgameTracker``.
* ``solve(F, starts; start_parameters, target_parameters)`` (src/solve.jl:447-526): one
  ``Result``; with a list of target parameters, the many-parameter solver (``many_solve``,
  src/solve.jl:747-880) — all targets in one batched GPU launch — returning
  ``transform_result(result, q)`` per target (default: the tuple ``(result, q)``), flattened on
  request.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from .systems import Poly, System
from .tracking import EndgameOptions, EndgameTracker, Result, TrackerOptions


class FiniteException(ValueError):
    """The system has fewer equations than variables (src/solve.jl:255, FiniteException(k))."""

    def __init__(self, k: int):
        super().__init__(f"FiniteException({k}): the solution set has dimension at least {k}")
        self.dim = k


class ParametricSystem:
    """Polynomial system F(x; p) with coefficients affine in the parameters p.

    For equation i: ``exponents[i]`` (terms × n int), ``c0[i]`` (terms,) complex and
    ``C[i]`` (terms × nparams) complex, coefficient_k(p) = c0[i][k] + C[i][k] · p.
    """

    def __init__(self, exponents, c0, C, nvars: int, nparams: int):
        self.exponents = [np.asarray(e, dtype=np.int32).reshape(-1, nvars) for e in exponents]
        self.c0 = [np.asarray(c, dtype=np.complex128).reshape(-1) for c in c0]
        self.C = [np.asarray(c, dtype=np.complex128).reshape(-1, nparams) for c in C]
        self.nvars = nvars
        self.nparams = nparams

    @staticmethod
    def from_polys(polys: Sequence[Poly], nvars: int, nparams: int) -> "ParametricSystem":
        """``polys`` are polynomials in nvars + nparams variables: the first nvars are the
        unknowns, the last nparams the parameters."""
        exps, c0s, Cs = [], [], []
        for i, p in enumerate(polys):
            if p.nvars != nvars + nparams:
                raise ValueError(f"equation {i}: expected {nvars + nparams} variables, got {p.nvars}")
            acc: dict = {}
            for k, v in p.terms.items():
                xe, pe = tuple(k[:nvars]), k[nvars:]
                dp = sum(pe)
                if dp > 1:
                    raise NotImplementedError(
                        "ParametricSystem holds coefficients affine in the parameters (a term of degree "
                        f"{dp} in the parameters in equation {i}); parametric_system() returns a "
                        "straight-line program for any other dependence")
                c = acc.setdefault(xe, [0j, np.zeros(nparams, dtype=np.complex128)])
                if dp == 0:
                    c[0] += v
                else:
                    c[1][int(np.argmax(pe))] += v
            ks = sorted(acc, key=lambda e: (-sum(e), tuple(-a for a in e)))
            exps.append(np.array(ks, dtype=np.int32).reshape(-1, nvars))
            c0s.append(np.array([acc[e][0] for e in ks], dtype=np.complex128))
            Cs.append(np.array([acc[e][1] for e in ks], dtype=np.complex128).reshape(-1, nparams))
        return ParametricSystem(exps, c0s, Cs, nvars, nparams)

    @staticmethod
    def coefficient_parameters(F: System) -> "ParametricSystem":
        """The family of all systems with F's support: every coefficient is a parameter (in
        equation order); F itself is the member at parameters = its coefficients."""
        total = sum(e.shape[0] for e in F.exponents)
        C, off = [], 0
        for e in F.exponents:
            Ci = np.zeros((e.shape[0], total), dtype=np.complex128)
            Ci[np.arange(e.shape[0]), off + np.arange(e.shape[0])] = 1.0
            C.append(Ci)
            off += e.shape[0]
        return ParametricSystem([e.copy() for e in F.exponents], [np.zeros(e.shape[0]) for e in F.exponents], C,
                                F.n, total)

    @property
    def n(self) -> int:
        return self.nvars

    @property
    def nequations(self) -> int:
        return len(self.exponents)

    @property
    def nparameters(self) -> int:
        return self.nparams

    def __call__(self, p) -> System:
        """The system with its parameters fixed to p (every term kept, also those whose
        coefficient vanishes at p, so that all fixings share one support)."""
        p = np.asarray(p, dtype=np.complex128).reshape(-1)
        if p.shape[0] != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters, got {p.shape[0]}")
        return System([e.copy() for e in self.exponents], [c0 + C @ p for c0, C in zip(self.c0, self.C)],
                      nvars=self.nvars)

    def evaluate(self, x, p):
        return self(p).evaluate(x)


def parametric_system(polys: Sequence[Poly], nvars: int, nparams: int):
    """``System(polys, variables, parameters)``: polynomials in nvars + nparams variables, the
    first nvars the unknowns. A ParametricSystem (term tables) when the parameters enter the
    coefficients affinely, else an ``slp.Program`` with parameters (monomials in x and p shared
    across equations)."""
    try:
        return ParametricSystem.from_polys(polys, nvars, nparams)
    except NotImplementedError:
        pass
    from .slp import Program, variables_and_parameters

    x, p = variables_and_parameters(nvars, nparams)
    v = list(x) + list(p)
    cache: dict = {}

    def mono(e):
        e = tuple(int(a) for a in e)
        if e not in cache:
            acc = None
            for j, k in enumerate(e):
                if k:
                    f = v[j] if k == 1 else v[j] ** k
                    acc = f if acc is None else acc * f
            cache[e] = acc
        return cache[e]

    outs, degs = [], []
    for poly in polys:
        if poly.nvars != nvars + nparams:
            raise ValueError(f"expected {nvars + nparams} variables, got {poly.nvars}")
        acc = None
        for e, c in poly.terms.items():
            m = mono(e)
            term = complex(c) if m is None else (m if c == 1 else complex(c) * m)
            acc = term if acc is None else acc + term
        outs.append(acc if acc is not None else 0.0)
        degs.append(max([sum(e[:nvars]) for e in poly.terms] + [1]))
    return Program(outs, degs)


class ParameterHomotopy:
    """H(x,t) = F(x; t p + (1-t) q) (src/homotopies/parameter_homotopy.jl:3-44). For a
    ParametricSystem (affine parameters) in the straight-line form the tracker runs: G = F(·; p),
    F = F(·; q), γ = 1; for an ``slp.Program`` with parameters, an ``SLPParameterHomotopy``."""

    def __new__(cls, F, start_parameters=None, target_parameters=None):
        from .slp import Program, SLPParameterHomotopy

        if isinstance(F, Program):
            return SLPParameterHomotopy(F, start_parameters, target_parameters)
        return super().__new__(cls)

    def __init__(self, F: ParametricSystem, start_parameters, target_parameters):
        m, n = F.nequations, F.n
        if m < n:
            raise FiniteException(n - m)
        if m > n:
            raise NotImplementedError("overdetermined systems are out of scope")
        self.system = F
        self.p = np.asarray(start_parameters, dtype=np.complex128).reshape(-1)
        self.q = np.asarray(target_parameters, dtype=np.complex128).reshape(-1)
        self.G = F(self.p)
        self.F = F(self.q)
        self.gamma = 1.0 + 0.0j

    @property
    def n(self) -> int:
        return self.system.n

    def parameters(self, p, q) -> "ParameterHomotopy":
        """New homotopy with parameters (p, q) (``parameters!``, :56-62); a tracker picks it up
        through ``set_homotopy``."""
        return ParameterHomotopy(self.system, p, q)


def parameter_homotopy(F, start_parameters=None, target_parameters=None,
                       generic_parameters=None, seed: Optional[int] = None):
    """src/solve.jl:233-260: missing parameters default to one generic complex vector. F: a
    ParametricSystem or an ``slp.Program`` with parameters."""
    if generic_parameters is None:
        rng = np.random.Generator(np.random.PCG64(seed))
        generic_parameters = (rng.standard_normal(F.nparams) + 1j * rng.standard_normal(F.nparams)) / np.sqrt(2)
    p = generic_parameters if start_parameters is None else start_parameters
    q = generic_parameters if target_parameters is None else target_parameters
    return ParameterHomotopy(F, p, q)


def _is_many(target_parameters) -> bool:
    if isinstance(target_parameters, (range, list, tuple)) and len(target_parameters) > 0:
        first = target_parameters[0]
        return not np.isscalar(first) or isinstance(target_parameters, range)
    a = np.asarray(target_parameters)
    return a.ndim == 2


def solve(F: ParametricSystem, starts, start_parameters, target_parameters, tracker_options=None,
          endgame_options=None, transform_result=None, transform_parameters=None, flatten: bool = False,
          precision: str = "fp64", step_control: str = "plain"):
    """solve(F, starts; start_parameters, target_parameters) (src/solve.jl:447-526) and, for a
    list of target parameters, the many-parameter solver (src/solve.jl:747-880) in one launch."""
    from .batch import BatchTracker

    to = tracker_options or TrackerOptions()
    to.precision = precision
    to.step_control = step_control
    eo = endgame_options or EndgameOptions()
    S = np.asarray(starts, dtype=np.complex128)
    if S.ndim == 1:
        S = S[None, :]
    if S.shape[1] != F.n:
        raise ValueError(f"start solutions must have {F.n} entries")
    if not _is_many(target_parameters):
        T = EndgameTracker(ParameterHomotopy(F, start_parameters, target_parameters), to, eo)
        return Result(T.track_batch(S), start_system=None)
    transform_result = transform_result or (lambda r, q: (r, q))
    transform_parameters = transform_parameters or (lambda q: q)
    targets = list(target_parameters)
    from .slp import Program

    if isinstance(F, Program):
        # one compiled program, retargeted per target parameters (two small device arrays)
        T = EndgameTracker(ParameterHomotopy(F, start_parameters, transform_parameters(targets[0])), to, eo)
        out = []
        for q in targets:
            T.set_homotopy(ParameterHomotopy(F, start_parameters, transform_parameters(q)))
            r = transform_result(Result(T.track_batch(S), start_system=None), q)
            if flatten:
                out.extend(r)
            else:
                out.append(r)
        return out
    Hs = [ParameterHomotopy(F, start_parameters, transform_parameters(q)) for q in targets]
    B = BatchTracker(Hs, to, eo, npaths=[S.shape[0]] * len(Hs))
    results = B.solve(starts=np.tile(S.reshape(-1), len(Hs)), start_system=None)
    out = []
    for R, q in zip(results, targets):
        r = transform_result(R, q)
        if flatten:
            out.extend(r)
        else:
            out.append(r)
    return out
