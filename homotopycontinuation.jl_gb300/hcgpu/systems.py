"""Polynomial systems in (support, coefficients) form and the total-degree start system.

A :class:`System` is the data ModelKit's ``support_coefficients`` yields for a square
polynomial system (src/model_kit/symbolic.jl:1130-1148, :1345-1348): for every equation an
exponent matrix (terms × variables) and a complex coefficient vector. The GPU tracker works
directly from these tables, so no symbolic engine is involved.

``Poly`` is a minimal sparse polynomial type (dict exponent-tuple → complex) used to write
systems such as ``(x - 10)**2`` or cyclic-n by hand.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np


class Poly:
    """Sparse multivariate polynomial over C in ``nvars`` variables."""

    __slots__ = ("nvars", "terms")

    def __init__(self, nvars: int, terms: dict | None = None):
        self.nvars = nvars
        self.terms = {} if terms is None else {k: complex(v) for k, v in terms.items() if v != 0}

    @staticmethod
    def var(i: int, nvars: int) -> "Poly":
        e = [0] * nvars
        e[i] = 1
        return Poly(nvars, {tuple(e): 1.0})

    @staticmethod
    def const(c, nvars: int) -> "Poly":
        return Poly(nvars, {(0,) * nvars: complex(c)})

    def _lift(self, o):
        return o if isinstance(o, Poly) else Poly.const(o, self.nvars)

    def __add__(self, o):
        o = self._lift(o)
        t = dict(self.terms)
        for k, v in o.terms.items():
            t[k] = t.get(k, 0) + v
        return Poly(self.nvars, t)

    __radd__ = __add__

    def __neg__(self):
        return Poly(self.nvars, {k: -v for k, v in self.terms.items()})

    def __sub__(self, o):
        return self + (-self._lift(o))

    def __rsub__(self, o):
        return self._lift(o) - self

    def __mul__(self, o):
        o = self._lift(o)
        t: dict = {}
        for k1, v1 in self.terms.items():
            for k2, v2 in o.terms.items():
                k = tuple(a + b for a, b in zip(k1, k2))
                t[k] = t.get(k, 0) + v1 * v2
        return Poly(self.nvars, t)

    __rmul__ = __mul__

    def __pow__(self, k: int):
        r = Poly.const(1.0, self.nvars)
        for _ in range(k):
            r = r * self
        return r

    def degree(self) -> int:
        return max((sum(k) for k in self.terms), default=0)


def variables(n: int):
    return [Poly.var(i, n) for i in range(n)]


@dataclass
class System:
    """Square polynomial system F: C^n → C^n in support/coefficient form.

    ``exponents[i]`` is an int array (terms_i × n), ``coefficients[i]`` a complex array
    (terms_i,) for equation i.
    """

    exponents: list
    coefficients: list
    nvars: int = field(default=0)

    def __post_init__(self):
        self.exponents = [np.asarray(e, dtype=np.int32).reshape(-1, self._n()) for e in self.exponents]
        self.coefficients = [np.asarray(c, dtype=np.complex128).reshape(-1) for c in self.coefficients]
        if not self.nvars:
            self.nvars = self.exponents[0].shape[1]
        if len(self.exponents) != len(self.coefficients):
            raise ValueError("exponents and coefficients must list the same equations")
        for e, c in zip(self.exponents, self.coefficients):
            if e.shape[0] != c.shape[0]:
                raise ValueError("each equation needs one coefficient per exponent row")
            if (e < 0).any():
                raise ValueError("exponents must be non-negative")

    def _n(self):
        if self.nvars:
            return self.nvars
        e = np.asarray(self.exponents[0])
        return e.shape[-1]

    @staticmethod
    def from_polys(polys) -> "System":
        n = polys[0].nvars
        exps, coefs = [], []
        for p in polys:
            ks = sorted(p.terms.keys(), key=lambda k: (-sum(k), tuple(-a for a in k)))
            exps.append(np.array(ks, dtype=np.int32).reshape(-1, n))
            coefs.append(np.array([p.terms[k] for k in ks], dtype=np.complex128))
        return System(exps, coefs, nvars=n)

    @property
    def n(self) -> int:
        return self.nvars

    @property
    def nequations(self) -> int:
        return len(self.exponents)

    def degrees(self):
        return [int(e.sum(axis=1).max()) if e.shape[0] else 0 for e in self.exponents]

    def is_homogeneous(self) -> bool:
        # src/total_degree.jl:48-61
        for e in self.exponents:
            d = e.sum(axis=1)
            if (d != d[0]).any():
                return False
        return True

    def term_arrays(self):
        """Flat (eq int32[T], exps int32[T×n], coef float64[T×2]) term tables."""
        eq = np.concatenate([np.full(e.shape[0], i, dtype=np.int32) for i, e in enumerate(self.exponents)])
        ex = np.ascontiguousarray(np.concatenate(self.exponents, axis=0), dtype=np.int32)
        c = np.concatenate(self.coefficients)
        cf = np.ascontiguousarray(np.stack([c.real, c.imag], axis=1), dtype=np.float64)
        return eq, ex, cf

    def evaluate(self, x):
        x = np.asarray(x, dtype=np.complex128)
        out = np.zeros(self.nequations, dtype=np.complex128)
        for i, (e, c) in enumerate(zip(self.exponents, self.coefficients)):
            out[i] = np.sum(c * np.prod(x[None, :] ** e, axis=1))
        return out


# --------------------------------------------------------------------------------------
# total-degree start system (src/total_degree.jl:32-117, :235-266)
# --------------------------------------------------------------------------------------
@dataclass
class TotalDegreeHomotopy:
    """H(x,t) = γ t G(x) + (1-t) F(x) with G_i = s_i (x_i^{D_i} - 1), s_i = max_j |c_ij|."""

    F: System
    G: System
    gamma: complex
    degrees: list
    scaling: np.ndarray

    @property
    def n(self):
        return self.F.n

    def bezout_number(self) -> int:
        return int(np.prod(self.degrees))


def total_degree_homotopy(F: System, gamma: complex) -> TotalDegreeHomotopy:
    n = F.n
    if F.nequations != n:
        raise NotImplementedError("only square systems are supported (overdetermined systems are out of scope)")
    if F.is_homogeneous():
        raise NotImplementedError("homogeneous systems (projective tracking) are out of scope")
    D = F.degrees()
    # src/total_degree.jl:62  scaling = maximum.(abs ∘ float, coeffs)
    scaling = np.array([np.max(np.abs(c)) for c in F.coefficients], dtype=np.float64)
    exps, coefs = [], []
    for i in range(n):
        e = np.zeros((2, n), dtype=np.int32)
        e[0, i] = D[i]
        exps.append(e)
        coefs.append(np.array([scaling[i], -scaling[i]], dtype=np.complex128))
    G = System(exps, coefs, nvars=n)
    return TotalDegreeHomotopy(F=F, G=G, gamma=complex(gamma), degrees=D, scaling=scaling)


def total_degree_start_solutions(degrees, index_range=None) -> np.ndarray:
    """Start solutions x_i = cis(2π k_i / D_i), product order with the first index fastest
    (src/total_degree.jl:240-262). Returns a (paths × n) complex array."""
    D = [int(d) for d in degrees]
    total = int(np.prod(D))
    idx = np.arange(total, dtype=np.int64) if index_range is None else np.asarray(index_range, dtype=np.int64)
    out = np.empty((idx.shape[0], len(D)), dtype=np.complex128)
    rem = idx.copy()
    for i, d in enumerate(D):
        k = rem % d
        rem //= d
        ang = (2 * np.pi) * k / d
        out[:, i] = np.cos(ang) + 1j * np.sin(ang)
    return out


def random_gamma(rng: np.random.Generator) -> complex:
    """γ = cis(2π u), u ~ U[0,1) (src/total_degree.jl:35, default argument)."""
    u = rng.random()
    return complex(np.cos(2 * np.pi * u), np.sin(2 * np.pi * u))


# --------------------------------------------------------------------------------------
# Seeded synthetic workloads
# --------------------------------------------------------------------------------------
def monomials_upto(n: int, d: int):
    """All exponent vectors of total degree ≤ d in n variables (degree-descending)."""
    out = []
    for deg in range(d, -1, -1):
        for comb in itertools.combinations_with_replacement(range(n), deg):
            e = [0] * n
            for j in comb:
                e[j] += 1
            out.append(tuple(e))
    return out


def complex_gaussian(rng, size):
    """i.i.d. standard complex Gaussian: re, im ~ N(0, 1/2)."""
    return (rng.normal(0.0, np.sqrt(0.5), size) + 1j * rng.normal(0.0, np.sqrt(0.5), size)).astype(np.complex128)


def dense_random_system(n: int, degrees, seed: int):
    """Dense system: equation i has every monomial of degree ≤ degrees[i] with complex
    Gaussian coefficients. Returns (System, γ) drawn from one seeded PCG64 stream."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if np.isscalar(degrees):
        degrees = [int(degrees)] * n
    exps, coefs = [], []
    for i in range(n):
        mons = monomials_upto(n, int(degrees[i]))
        exps.append(np.array(mons, dtype=np.int32))
        coefs.append(complex_gaussian(rng, len(mons)))
    gamma = random_gamma(rng)
    return System(exps, coefs, nvars=n), gamma


def sparse_random_system(n: int, nterms: int, maxdeg: int, seed: int):
    """Sparse system: each equation has ``nterms`` distinct random monomials of total degree
    ≤ maxdeg (at least one of degree exactly maxdeg) plus a constant term."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pool = [m for m in monomials_upto(n, maxdeg) if sum(m) > 0]
    top = [k for k, m in enumerate(pool) if sum(m) == maxdeg]
    exps, coefs = [], []
    for i in range(n):
        first = int(rng.choice(top))
        rest = [k for k in range(len(pool)) if k != first]
        pick = [first] + list(rng.choice(rest, size=nterms - 1, replace=False))
        e = np.array([pool[k] for k in pick] + [(0,) * n], dtype=np.int32)
        exps.append(e)
        coefs.append(complex_gaussian(rng, e.shape[0]))
    gamma = random_gamma(rng)
    return System(exps, coefs, nvars=n), gamma


def uneven_instances(count: int, seed: int):
    """Batch of independent dense instances: n ~ U{3..8}, each equation degree ~ U{2,3}."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(count):
        n = int(rng.integers(3, 9))
        degs = [int(d) for d in rng.integers(2, 4, size=n)]
        sub_seed = int(rng.integers(0, 2**62))
        F, g = dense_random_system(n, degs, sub_seed)
        out.append((F, g))
    return out


def cyclic(n: int) -> System:
    """cyclic-n: Σ_j Π_{k=j}^{j+m} z_{k mod n} for m = 0..n-2, and Π z - 1."""
    z = variables(n)
    eqs = []
    for m in range(n - 1):
        acc = Poly.const(0.0, n)
        for j in range(n):
            p = Poly.const(1.0, n)
            for k in range(j, j + m + 1):
                p = p * z[k % n]
            acc = acc + p
        eqs.append(acc)
    p = Poly.const(1.0, n)
    for v in z:
        p = p * v
    eqs.append(p - 1.0)
    return System.from_polys(eqs)
