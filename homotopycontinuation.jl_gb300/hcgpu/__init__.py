"""hcgpu — GB300-native path tracking with the API of HomotopyContinuation.jl's
total-degree hot path. See include/hcgpu.h for the C ABI."""
from .systems import (
    Poly,
    System,
    TotalDegreeHomotopy,
    complex_gaussian,
    cyclic,
    dense_random_system,
    monomials_upto,
    random_gamma,
    sparse_random_system,
    total_degree_homotopy,
    total_degree_start_solutions,
    uneven_instances,
    variables,
)
from . import slp
from .batch import BatchTracker, autotune, autotune_unit_paths, solve_batch
from .certification import CertificationResult, SolutionCertificate, certify
from .io import read_parameters, read_solutions, write_parameters, write_solutions
from .monodromy import MonodromyResult, find_start_pair, monodromy_solve
from .parameters import FiniteException, ParameterHomotopy, ParametricSystem, parameter_homotopy, parametric_system
from .polyhedral_homotopy import (MixedCell, PolyhedralStartSolutions, PolyhedralTracker, fine_mixed_cells, mixed_volume,
                         paths_to_track, polyhedral, solve_binomial)
from .tracking import (
    ENDGAME_CODES,
    TRACKER_CODES,
    EndgameOptions,
    EndgameTracker,
    PathResult,
    Result,
    Tracker,
    TrackerOptions,
    TrackerResult,
    make_options,
    multiplicities,
    nat_infinity,
    nfailed,
    nnonsingular,
    nsingular,
    solve,
    total_degree,
    track,
)

__all__ = [n for n in dir() if not n.startswith("_")]
