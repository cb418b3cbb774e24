"""Generate tests/golden/kat_systems.json from HomotopyContinuation.jl's own test files.

The known-answer systems, fixed γ values and expected counts of the reference's endgame,
EndgameTracker and valuation tests are read as text from the reference checkout and turned
into term tables (exponent rows + complex coefficients). Run in a container that has the
reference sources:

    python tests/golden/make_fixtures.py /path/to/HomotopyContinuation.jl

The JSON is committed; the tests never read the reference checkout.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "homotopycontinuation.jl_gb300"))

from hcgpu.systems import Poly, System, variables  # noqa: E402


def julia_to_python(expr: str) -> str:
    e = expr.replace("\n", " ")
    e = e.replace("^", "**")
    e = re.sub(r"(\d)([a-zA-Z(])", r"\1*\2", e)  # implicit multiplication 3x, 2(, 1.3im
    e = re.sub(r"\bim\b", "1j", e)
    return e


def to_system(exprs, names):
    vs = variables(len(names))
    env = dict(zip(names, vs))
    polys = [eval(julia_to_python(e), {}, env) for e in exprs]
    polys = [p if isinstance(p, Poly) else Poly.const(p, len(names)) for p in polys]
    S = System.from_polys(polys)
    return {"n": S.n, "exponents": [e.tolist() for e in S.exponents],
            "coefficients": [[[c.real, c.imag] for c in cs] for cs in S.coefficients]}


def to_param_system(exprs, names, params):
    """Polynomials in the unknowns `names` and parameters `params` as one term table over
    names + params (the test builds a ParametricSystem from it)."""
    allv = list(names) + list(params)
    vs = variables(len(allv))
    env = dict(zip(allv, vs))
    polys = [eval(julia_to_python(e), {}, env) for e in exprs]
    eqs = []
    for p in polys:
        ks = sorted(p.terms)
        eqs.append({"exponents": [list(k) for k in ks],
                    "coefficients": [[p.terms[k].real, p.terms[k].imag] for k in ks]})
    return {"nvars": len(names), "nparams": len(params), "equations": eqs}


def split_top_level(s: str):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [o.strip() for o in out if o.strip()]


def main(ref):
    test = os.path.join(ref, "test")
    eg = open(os.path.join(test, "endgame_tracker_test.jl")).read()
    en = open(os.path.join(test, "endgame_test.jl")).read()
    val = open(os.path.join(test, "valuation_test.jl")).read()
    out = {"source": "HomotopyContinuation.jl test/endgame_tracker_test.jl, test/endgame_test.jl, "
                     "test/valuation_test.jl, test/tracker_test.jl, test/solve_test.jl, "
                     "test/certification_test.jl"}

    # EndgameTracker test: 2×2 quadrics, γ = 1.3im + 0.4
    m = re.search(r"f = \[(2\.3 \* x\^2.*?)\]\n\s*tracker, starts = total_degree\(System\(f\); gamma = ([^)]*)\)", eg)
    out["quadrics_2x2"] = {**to_system(split_top_level(m.group(1)), ["x", "y"]),
                           "gamma": list(map(float, [complex(eval(julia_to_python(m.group(2)))).real,
                                                      complex(eval(julia_to_python(m.group(2)))).imag])),
                           "expect": {"codes": ["success", "success", "at_infinity", "at_infinity"],
                                      "valuation_at_infinity": [-1.0, -1.0]}}
    # winding number family a-coefficients
    m = re.search(r'Winding Number Family.*?a = \[([^\]]*)\]', en, re.S)
    a = [float(v) for v in m.group(1).split(",")]
    out["winding_family_a"] = a
    # Mohab system + fixed γ; the reference orders the variables as System(F, [x, z, y])
    blk = en[en.index('@testset "Mohab"'):]
    m = re.search(r"F = \[(.*?)\n\s*\]\n", blk, re.S)
    eqs = split_top_level(m.group(1))
    g = re.search(r"γ = ([-0-9.e]+) \+ ([0-9.e]+)im", blk)
    out["mohab"] = {**to_system(eqs, ["x", "z", "y"]), "gamma": [float(g.group(1)), float(g.group(2))],
                    "expect": {"nnonsingular": int(re.search(r"nnonsingular\(res\) == (\d+)", blk).group(1))}}
    # multiplicity KATs: "Hyperbolic - 6,6" (dehomogenised at y = 1; 12 paths with winding
    # number 3, 2 singular results of multiplicity 6) and "Singular 1" (z = 1; one singular
    # solution of multiplicity 3 and one nonsingular solution)
    blk = en[en.index('@testset "Hyperbolic - 6,6"'):en.index('@testset "Singular 1"')]
    m = re.search(r"F = \[\n(.*?)\n\s*\]\n", blk, re.S)
    rows = [r.strip() for r in m.group(1).split("\n") if r.strip()]
    rows = [r.replace("y", "1") for r in rows]
    out["hyperbolic_6_6"] = {**to_system(rows, ["x", "z"]), "expect": {
        "n_winding": int(re.search(r"winding_number == (\d+), path_results\(res\)\) == (\d+)", blk).group(2)),
        "winding_number": int(re.search(r"winding_number == (\d+)", blk).group(1)),
        "nresults": int(re.search(r"nresults\(res\) == (\d+)", blk).group(1)),
        "nsingular": int(re.search(r"nsingular\(res\) == (\d+)", blk).group(1)),
        "multiplicity": int(re.search(r"multiplicity\(r\) == (\d+)", blk).group(1))}}
    blk = en[en.index('@testset "Singular 1"'):en.index('@testset "Wilkinson')]
    m = re.search(r"F = \[\n(.*?)\n\s*\]\n", blk, re.S)
    rows = split_top_level(m.group(1).replace("\n", " "))
    rows = [re.sub(r"\bz\b", "1", r) for r in rows]
    out["singular_1"] = {**to_system(rows, ["x", "y"]), "expect": {
        "nsingular": int(re.search(r"nsingular\(result\) == (\d+)", blk).group(1)),
        "nresults_nonsingular": int(re.search(r"only_nonsingular = true\) == (\d+)", blk).group(1))}}
    # cyclic-7 expected count
    out["cyclic7"] = {"expect": {"nsolutions": int(re.search(r"cyclic\(7\).*?nsolutions\(res\) == (\d+)", en, re.S).group(1))}}
    # valuation example 3 (endgame side) system and targets
    m = re.search(r'Example 3.*?a = \[([^\]]*)\]', val, re.S)
    out["valuation_example3_a"] = [float(v) for v in m.group(1).split(",")]
    # parameter homotopy (test/tracker_test.jl: Tracker(ParameterHomotopy(F, [1, 0], [2, 4])))
    tr = open(os.path.join(test, "tracker_test.jl")).read()
    m = re.search(r"F = System\(\[(x\^2 - a, x \* y - a \+ b)\], \[x, y\], \[a, b\]\)", tr)
    h = re.search(r"ParameterHomotopy\(mode\(F\), \[([^\]]*)\], \[([^\]]*)\]\)", tr)
    st = re.search(r"s = \[([^\]]*)\]\n\s*res = track\(tracker, s, 1, 0\)", tr)
    steps = re.search(r"@test steps\(res\) ≤ (\d+)", tr)
    sol = re.search(r"@test solution\(res\) ≈ \[sqrt\((\d+)\), -sqrt\((\d+)\)\]", tr)
    out["parameter_tracker"] = {
        **to_param_system(split_top_level(m.group(1)), ["x", "y"], ["a", "b"]),
        "start_parameters": [float(v) for v in h.group(1).split(",")],
        "target_parameters": [float(v) for v in h.group(2).split(",")],
        "start": [float(v) for v in st.group(1).split(",")],
        "expect": {"max_steps": int(steps.group(1)),
                   "solution": [float(sol.group(1)) ** 0.5, -float(sol.group(2)) ** 0.5]}}
    # solve (parameter homotopy): nsolutions == 1 (test/solve_test.jl)
    sv = open(os.path.join(test, "solve_test.jl")).read()
    blk = sv[sv.index('@testset "solve (parameter homotopy)"'):]
    n1 = re.search(r"solve\(F, \[s\]; start_parameters = \[1, 0\], target_parameters = \[2, 4\]\)\n"
                   r"\s*@test nsolutions\(res\) == (\d+)", blk)
    fe = re.search(r"F = System\(\[(x\^2 - a)\], \[x, y\], \[a, b\]\)\n\s*s = \[1, 1\]\n\s*"
                   r"@test_throws FiniteException\((\d+)\)", blk)
    out["parameter_solve"] = {"expect": {"nsolutions": int(n1.group(1)), "finite_exception_dim": int(fe.group(2))},
                              "underdetermined": to_param_system([fe.group(1)], ["x", "y"], ["a", "b"])}
    # Beyond Polyhedral Homotopy Example: 2 successes, 2 at infinity (test/endgame_test.jl)
    blk = en[en.index('@testset "Beyond Polyhedral Homotopy Example"'):]
    fb = re.search(r"f = \[(.*?)\]\n", blk).group(1)
    out["beyond_polyhedral"] = {**to_system(split_top_level(fb), ["x", "y"]), "expect": {
        "success": int(re.search(r"count\(is_success, res\) == (\d+)", blk).group(1)),
        "at_infinity": int(re.search(r"count\(is_at_infinity, res\) == (\d+)", blk).group(1))}}
    # Tracker on a straight-line homotopy with a given start system (test/tracker_test.jl)
    blk = tr[tr.index('@testset "Straight Line Homotopy"'):]
    Fs = re.search(r"F = System\(\[(.*?)\], \[x, y\]\)", blk).group(1)
    gm = re.search(r"G = System\(\(([^)]*)\) \.\* \[(.*?)\], \[x, y\]\)", blk)
    starts = re.search(r"S = \[\[(.*?)\], \[(.*?)\]\]", blk)
    bad = re.search(r"is_invalid_startvalue\(track\(tracker, \[(.*?)\], 1, 0\)\)", blk)
    scale = complex(eval(julia_to_python(gm.group(1))))
    G = to_system(split_top_level(gm.group(2)), ["x", "y"])
    G["coefficients"] = [[[(complex(*c) * scale).real, (complex(*c) * scale).imag] for c in cs]
                         for cs in G["coefficients"]]
    out["straight_line_tracker"] = {"F": to_system(split_top_level(Fs), ["x", "y"]), "G": G,
                                    "starts": [[float(v) for v in starts.group(1).split(",")],
                                               [float(v) for v in starts.group(2).split(",")]],
                                    "invalid_start": [float(v) for v in bad.group(1).split(",")],
                                    "expect": {"starts": "success", "invalid_start": "terminated_invalid_startvalue"}}
    # solve (DynamicPolynomials): nsolutions == 18 (test/solve_test.jl)
    blk = sv[sv.index('@testset "solve (DynamicPolynomials)"'):]
    d1 = re.search(r"f₁ = (.*)\n", blk).group(1).strip()
    d2p = re.search(r"f₂ = (.*)\n", blk).group(1).strip()
    out["dynamic_polynomials_18"] = {**to_system([d1, d2p], ["x", "y"]), "expect": {
        "nsolutions": int(re.search(r"result = solve\(\[f₁, f₂\]\)\n\s*@test nsolutions\(result\) == (\d+)",
                                    blk).group(1))}}
    # certification (test/certification_test.jl "Simple 1")
    ce = open(os.path.join(test, "certification_test.jl")).read()
    blk = ce[ce.index('@testset "Simple 1'):]
    f1 = re.search(r"f₁ = (.*)\n", blk).group(1).strip()
    f2 = re.search(r"f₂ = (.*)\n", blk).group(1).strip()
    num = lambda pat: int(re.search(pat, blk).group(1))
    d2 = blk[blk.index("# Double solutions"):]
    num2 = lambda pat: int(re.search(pat, d2).group(1))
    out["certification_simple"] = {
        **to_system([f1, f2], ["x", "y"]),
        "expect": {"nnonsingular": num(r"@test nnonsingular\(result\) == (\d+)"),
                   "ncertified": num(r"@test ncertified\(cert\) == (\d+)"),
                   "ndistinct_certified": num(r"@test ndistinct_certified\(cert\) == (\d+)"),
                   "nreal_certified": num(r"@test nreal_certified\(cert\) == (\d+)"),
                   "ncomplex_certified": num(r"@test ncomplex_certified\(cert\) == (\d+)"),
                   "doubled": {"ncertified": num2(r"@test ncertified\(cert\) == (\d+)"),
                               "ndistinct_certified": num2(r"@test ndistinct_certified\(cert\) == (\d+)"),
                               "nreal_certified": num2(r"@test nreal_certified\(cert\) == (\d+)"),
                               "ndistinct_real_certified": num2(r"@test ndistinct_real_certified\(cert\) == (\d+)")}}}
    with open(os.path.join(HERE, "kat_systems.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "kat_systems.json"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path of a HomotopyContinuation.jl checkout>")
    main(sys.argv[1])
