"""Bertini-format solution and parameter files (src/utils.jl:1-125; test/utils_test.jl)."""
import numpy as np

import hcgpu as hc


def test_solutions_round_trip_and_format(tmp_path):
    p = tmp_path / "sols.txt"
    hc.write_solutions(p, [[1, 1], [-1, 2]])
    # the layout of the reference's docstring example
    assert p.read_text() == "2\n\n1 0\n1 0\n\n-1 0\n2 0\n"
    assert [list(s) for s in hc.read_solutions(p)] == [[1, 1], [-1, 2]]
    rng = np.random.default_rng(0)
    S = [rng.normal(size=3) + 1j * rng.normal(size=3) for _ in range(5)]
    hc.write_solutions(p, S)
    R = hc.read_solutions(p)
    assert len(R) == 5 and all((a == b).all() for a, b in zip(R, S))


def test_parameters_round_trip_and_format(tmp_path):
    p = tmp_path / "params.txt"
    hc.write_parameters(p, [2.0, -3.2 + 2j])
    assert p.read_text() == "2\n\n2.0 0.0\n-3.2 2.0\n"
    assert list(hc.read_parameters(p)) == [2.0, -3.2 + 2j]
