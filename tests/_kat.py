"""Known-answer systems of the reference test suite (tests/golden/kat_systems.json)."""
import json
import os

import numpy as np

import hcgpu as hc

_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kat_systems.json")
KAT = json.load(open(_PATH))


def system(name):
    d = KAT[name]
    return hc.System([np.array(e, dtype=np.int32) for e in d["exponents"]],
                     [np.array([complex(*c) for c in cs]) for cs in d["coefficients"]], nvars=d["n"])


def system_of(d):
    """A System from a fixture dictionary (n, exponents, coefficients)."""
    return hc.System([np.array(e, dtype=np.int32) for e in d["exponents"]],
                     [np.array([complex(*c) for c in cs]) for cs in d["coefficients"]], nvars=d["n"])


def straight_line_homotopy():
    """The Tracker test's straight-line homotopy t G + (1 - t) F with its own start system G
    (no total-degree scaling; γ = 1)."""
    d = KAT["straight_line_tracker"]
    F, G = system_of(d["F"]), system_of(d["G"])
    return hc.systems.TotalDegreeHomotopy(F=F, G=G, gamma=1.0 + 0j, degrees=[2, 1], scaling=np.ones(2))


def gamma(name):
    return complex(*KAT[name]["gamma"])


def winding_family(d):
    a = KAT["winding_family_a"]
    x, y = hc.variables(2)
    f1 = (a[0] * x**d + a[1] * y) * (a[2] * x + a[3] * y) + 1
    f2 = (a[0] * x**d + a[1] * y) * (a[4] * x + a[5] * y) + 1
    return hc.System.from_polys([f1, f2])


def parametric_system(d):
    """ParametricSystem from a term table over unknowns + parameters (fixtures' format)."""
    nv, npar = d["nvars"], d["nparams"]
    polys = []
    for eq in d["equations"]:
        polys.append(hc.Poly(nv + npar, {tuple(e): complex(*c) for e, c in zip(eq["exponents"], eq["coefficients"])}))
    return hc.ParametricSystem.from_polys(polys, nv, npar)


def term_lists(S):
    """Per equation [(exponent tuple, complex coefficient)] of a System."""
    return [[(tuple(int(v) for v in e), complex(c)) for e, c in zip(E, Cs)] for E, Cs in zip(S.exponents, S.coefficients)]


def jacobian(S, x):
    n = S.n
    J = np.zeros((n, n), dtype=np.complex128)
    for i, (E, Cs) in enumerate(zip(S.exponents, S.coefficients)):
        for e, c in zip(E, Cs):
            for j in range(n):
                if e[j] > 0:
                    d = e.copy()
                    d[j] -= 1
                    J[i, j] += c * e[j] * np.prod(x ** d)
    return J
