"""certify(F, solutions) (src/certification.jl:691-745) on the GPU.

Every candidate gets a Krawczyk certificate from ``hc_certify`` (csrc/hc_certify.cu): a polydisc
B = B(center, radius) that provably contains exactly one solution, which lies in the smaller
polydisc K = B(enclosure center, enclosure), and whether that solution is provably real or
non-real. Candidates that FP64 balls cannot certify are retried with double-word centres
(``precision`` 106), as the reference retries with Arb balls. Distinctness is decided here from the certificates: two certified candidates name the
same solution if one's K lies in the other's B (that B holds a single solution), and different
solutions if their K's are disjoint; pairs where neither holds are counted as distinct and
reported in ``nundecided_pairs``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .systems import System, total_degree_homotopy
from .tracking import Result, _Handle, make_options


@dataclass
class SolutionCertificate:
    solution_candidate: np.ndarray
    certified: bool
    real: bool           # provably real
    complex: bool        # provably non-real
    center: np.ndarray   # box centre (candidate after one Newton step)
    radius: float
    enclosure_center: np.ndarray
    enclosure: float
    index: int
    precision: int = 53  # bits of the centres that decided (106: the double-word pass)

    def is_certified(self):
        return self.certified

    def is_real(self):
        return self.real


@dataclass
class CertificationResult:
    """src/certification.jl CertificationResult: certificates and (distinct) counts."""

    certificates: list
    classes: list = field(default_factory=list)  # class id per certificate (-1: not certified)
    nundecided_pairs: int = 0

    def ncertified(self):
        return sum(c.certified for c in self.certificates)

    def nreal_certified(self):
        return sum(c.certified and c.real for c in self.certificates)

    def ncomplex_certified(self):
        return sum(c.certified and c.complex for c in self.certificates)

    def _reps(self):
        seen = {}
        for c, k in zip(self.certificates, self.classes):
            if k >= 0 and k not in seen:
                seen[k] = c
        return list(seen.values())

    def ndistinct_certified(self):
        return len(self._reps())

    def ndistinct_real_certified(self):
        return sum(c.real for c in self._reps())

    def ndistinct_complex_certified(self):
        return sum(c.complex for c in self._reps())

    def __repr__(self):
        return (f"CertificationResult: {len(self.certificates)} candidates, {self.ncertified()} certified "
                f"({self.nreal_certified()} real, {self.ncomplex_certified()} complex), "
                f"{self.ndistinct_certified()} distinct ({self.ndistinct_real_certified()} real, "
                f"{self.ndistinct_complex_certified()} complex)")


def _classes(certs):
    """Union-find over proven duplicates (K_a ⊂ B_b); candidates swept by the first coordinate."""
    idx = [i for i, c in enumerate(certs) if c.certified]
    parent = {i: i for i in idx}

    def find(i):
        while parent[i] != i:
            parent[i] = parent[parent[i]]
            i = parent[i]
        return i

    if not idx:
        return [-1] * len(certs), 0
    key = np.array([certs[i].enclosure_center[0].real for i in idx])
    order = np.argsort(key)
    reach = max(certs[i].radius + certs[i].enclosure for i in idx)
    undecided = 0
    for a_pos in range(len(order)):
        a = idx[order[a_pos]]
        ca = certs[a]
        for b_pos in range(a_pos + 1, len(order)):
            b = idx[order[b_pos]]
            cb = certs[b]
            if cb.enclosure_center[0].real - ca.enclosure_center[0].real > 2 * reach:
                break
            # disjoint enclosures: different solutions
            gap = np.abs(ca.enclosure_center - cb.enclosure_center) - (ca.enclosure + cb.enclosure)
            if (gap > 0).any():
                continue
            inside_b = (np.abs(ca.enclosure_center - cb.center) + ca.enclosure < cb.radius).all()
            inside_a = (np.abs(cb.enclosure_center - ca.center) + cb.enclosure < ca.radius).all()
            if inside_a or inside_b:
                parent[find(a)] = find(b)
            else:
                undecided += 1
    classes = [-1] * len(certs)
    for i in idx:
        classes[i] = find(i)
    return classes, undecided


def certify(F: System, solutions) -> CertificationResult:
    """Certify approximate solutions (a list of vectors or a Result) of the square system F."""
    if isinstance(solutions, Result):
        cands = [r.solution for r in solutions.path_results if r.is_success()]
    else:
        cands = list(solutions)
    S = np.ascontiguousarray(np.array(cands, dtype=np.complex128).reshape(len(cands), F.n))
    real_coef = all(np.all(np.imag(c) == 0) for c in F.coefficients)
    h = _Handle(make_options())
    h.set_homotopy(total_degree_homotopy(F, 1.0 + 0j))  # only F (H at t = 0) is certified
    out = np.zeros(len(S), dtype=_lib.CERT_DTYPE)
    centers = np.zeros_like(S)
    encl = np.zeros_like(S)
    P = _lib.ptr
    if len(S):
        _lib.check(h.L.hc_certify(h.h, len(S), P(S), 1 if real_coef else 0, P(out), P(centers), P(encl)), h.h)
    certs = [SolutionCertificate(solution_candidate=S[k].copy(), certified=bool(out["certified"][k]),
                                 real=bool(out["realness"][k] == 1), complex=bool(out["realness"][k] == 2),
                                 center=centers[k].copy(), radius=float(out["radius"][k]),
                                 enclosure_center=encl[k].copy(), enclosure=float(out["enclosure"][k]), index=k,
                                 precision=int(out["precision"][k]))
             for k in range(len(S))]
    classes, undecided = _classes(certs)
    return CertificationResult(certs, classes, undecided)


def main(argv=None):
    """python -m hcgpu.certification [--n 10] [--degree 3] [--seed 0]: solve a seeded dense
    system by total degree on the GPU and certify every nonsingular solution."""
    import argparse
    import json
    import time

    from .systems import dense_random_system
    from .tracking import TrackerOptions, solve

    ap = argparse.ArgumentParser(description=main.__doc__.split("\n")[0])
    ap.add_argument("--n", type=int, default=10)
    ap.add_argument("--degree", type=int, default=3)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    F, g = dense_random_system(a.n, a.degree, seed=a.seed)
    t = time.time()
    R = solve(F, gamma=g, precision="mixed", step_control="learned")
    ts = time.time() - t
    S = [r.solution for r in R.path_results if r.is_success() and not r.is_singular()]
    certify(F, S[:16])  # first launch (module load, set-up)
    t = time.time()
    C = certify(F, S)
    tc = time.time() - t
    print(json.dumps({"system": f"{a.n} dense polynomials of degree {a.degree} (seed {a.seed})",
                      "nonsingular": len(S), "certified": C.ncertified(), "distinct": C.ndistinct_certified(),
                      "undecided_pairs": C.nundecided_pairs, "solve_seconds": ts, "certify_seconds": tc,
                      "certified_per_second": C.ncertified() / tc}))


if __name__ == "__main__":
    main()
