"""Solution and parameter files in Bertini's plain-text format (src/utils.jl:1-125).

    write_solutions(path, solutions)   # count, blank line, then per solution "re im" lines
    read_solutions(path)               # list of complex vectors
    write_parameters(path, p)          # count, blank line, "re im" lines
    read_parameters(path)
"""
from __future__ import annotations

from typing import Sequence

import numpy as np


def _pairs(values):
    """(real, imag) text of each value: integer inputs as integers, others as shortest
    round-trip floats (the way writedlm prints Int and Float64)."""
    a = np.asarray(values).reshape(-1)
    if np.issubdtype(a.dtype, np.integer):
        return [(str(int(v)), "0") for v in a]
    a = a.astype(np.complex128)
    return [(repr(float(z.real)), repr(float(z.imag))) for z in a]


def write_solutions(path, solutions: Sequence[Sequence[complex]]) -> None:
    """The number of solutions, then each solution after a blank line, one coordinate per line
    as "real imag" (src/utils.jl:35-44)."""
    with open(path, "w") as f:
        f.write(f"{len(solutions)}\n")
        for s in solutions:
            f.write("\n")
            for re, im in _pairs(s):
                f.write(f"{re} {im}\n")


def read_solutions(path):
    """Solutions written by write_solutions (src/utils.jl:63-78)."""
    lines = open(path).read().split("\n")
    count = int(float(lines[0].split()[0]))
    out, cur = [], []
    for line in lines[2:]:
        parts = line.split()
        if not parts:
            if cur:
                out.append(np.array(cur, dtype=np.complex128))
                cur = []
            continue
        cur.append(complex(float(parts[0]), float(parts[1]) if len(parts) > 1 else 0.0))
    if cur:
        out.append(np.array(cur, dtype=np.complex128))
    if len(out) != count:
        raise ValueError(f"{path}: header announces {count} solutions, found {len(out)}")
    return out


def write_parameters(path, p: Sequence[complex]) -> None:
    """The number of values, a blank line, then one "real imag" line each (src/utils.jl:103-108)."""
    pairs = _pairs(p)
    with open(path, "w") as f:
        f.write(f"{len(pairs)}\n\n")
        for re, im in pairs:
            f.write(f"{re} {im}\n")


def read_parameters(path):
    """Parameters written by write_parameters (src/utils.jl:121-125)."""
    rows = [line.split() for line in open(path).read().split("\n") if line.split()]
    n = int(float(rows[0][0]))
    return np.array([complex(float(r[0]), float(r[1])) for r in rows[1:n + 1]], dtype=np.complex128)
