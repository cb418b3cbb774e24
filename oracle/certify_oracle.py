"""CPU oracle for the Krawczyk certificates (test infrastructure only).

An independent restatement of the Krawczyk test (Moore 1977; as in the reference's
src/certification.jl, after Breiding, Rose and Timme 2020) in EXACT rational interval
arithmetic: every floating-point input is converted to a Fraction, complex numbers are
rectangles [re_lo, re_hi] + i [im_lo, im_hi], and all operations are exact, so the only
over-approximation is the interval dependency of the Krawczyk operator itself. For a candidate
x̃, box radius r and point matrix Y ≈ J(x̃)⁻¹ (both supplied by the caller, as the GPU kernel
computes them):

    K = x̃ − Y F(x̃) + (I − Y J(X)) (X − x̃),   X = x̃ + [−r, r] + i[−r, r] per coordinate,

certified iff K ⊂ int X; real iff, with real coefficients, conj(K) ⊂ int X; non-real iff some
coordinate of K does not meet the real axis. Slow (pure Python rationals): for small systems.
"""
from __future__ import annotations

from fractions import Fraction as Q


class I:
    """Closed rational interval."""

    __slots__ = ("lo", "hi")

    def __init__(self, lo, hi=None):
        self.lo = Q(lo)
        self.hi = Q(lo if hi is None else hi)

    def __add__(self, o):
        o = o if isinstance(o, I) else I(o)
        return I(self.lo + o.lo, self.hi + o.hi)

    def __sub__(self, o):
        o = o if isinstance(o, I) else I(o)
        return I(self.lo - o.hi, self.hi - o.lo)

    def __neg__(self):
        return I(-self.hi, -self.lo)

    def __mul__(self, o):
        o = o if isinstance(o, I) else I(o)
        p = [self.lo * o.lo, self.lo * o.hi, self.hi * o.lo, self.hi * o.hi]
        return I(min(p), max(p))

    def inside(self, o) -> bool:  # strictly inside o
        return o.lo < self.lo and self.hi < o.hi

    def contains0(self) -> bool:
        return self.lo <= 0 <= self.hi


class C:
    """Complex rectangle."""

    __slots__ = ("re", "im")

    def __init__(self, re, im=None):
        self.re = re if isinstance(re, I) else I(re)
        self.im = (im if isinstance(im, I) else I(im)) if im is not None else I(0)

    @staticmethod
    def of(z):
        z = complex(z)
        return C(I(Q(z.real)), I(Q(z.imag)))

    def __add__(self, o):
        return C(self.re + o.re, self.im + o.im)

    def __sub__(self, o):
        return C(self.re - o.re, self.im - o.im)

    def __mul__(self, o):
        return C(self.re * o.re - self.im * o.im, self.re * o.im + self.im * o.re)

    def conj(self):
        return C(self.re, -self.im)


def _poly(terms, X, n):
    """Σ c · Π X_j^e_j for terms [(exponent tuple, complex coefficient)]."""
    acc = C(0)
    for e, c in terms:
        m = C.of(c)
        for j in range(n):
            for _ in range(e[j]):
                m = m * X[j]
        acc = acc + m
    return acc


def _deriv(terms, j):
    out = []
    for e, c in terms:
        if e[j] > 0:
            d = list(e)
            d[j] -= 1
            out.append((tuple(d), complex(c) * e[j]))
    return out


def krawczyk(system, x, r, Y, real_coefficients):
    """system: per equation a list of (exponent tuple, complex coefficient); x: candidate (n
    complex); r: box radius (float); Y: n×n complex point matrix. Returns
    (certified, realness) with realness 1 real, 2 non-real, 0 undecided."""
    n = len(x)
    xc = [C.of(v) for v in x]
    R = I(-Q(r), Q(r))
    X = [C(xc[j].re + R, xc[j].im + R) for j in range(n)]
    F = [_poly(eq, xc, n) for eq in system]
    J = [[_poly(_deriv(eq, j), X, n) for j in range(n)] for eq in system]
    Yc = [[C.of(Y[i][j]) for j in range(n)] for i in range(n)]
    K = []
    for i in range(n):
        yf = C(0)
        for j in range(n):
            yf = yf + Yc[i][j] * F[j]
        s = C(0)
        for j in range(n):
            mij = C(1 if i == j else 0)
            for q in range(n):
                mij = mij - Yc[i][q] * J[q][j]
            s = s + mij * C(R, R)
        K.append(xc[i] - yf + s)
    certified = all(K[i].re.inside(X[i].re) and K[i].im.inside(X[i].im) for i in range(n))
    realness = 0
    if certified:
        if real_coefficients and all(K[i].conj().re.inside(X[i].re) and K[i].conj().im.inside(X[i].im)
                                     for i in range(n)):
            realness = 1
        elif any(not K[i].im.contains0() for i in range(n)):
            realness = 2
    return certified, realness
