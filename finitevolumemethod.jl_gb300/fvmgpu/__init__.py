"""fvmgpu: GB300-native vertex-centred finite-volume hot path with FiniteVolumeMethod.jl's API.

The compute path is libfvmgpu.so (hand-written sm_103a CUDA kernels behind the C ABI of
include/fvm_gpu.h); this package is the host-side mirror of the reference interface.
"""
from .meshes import (Triangulation, triangulate_rectangle, triangulate_annulus, triangulate_disk, triangulate_points,
                     disjoint_union)
from .api import (ConditionType, Neumann, Dudt, Dirichlet, Constrained, ParametrisedFunction, BoundaryConditions,
                  InternalConditions, Conditions, TriangleProperties, FVMGeometry, FVMProblem, fvm_eqs,
                  update_dirichlet_nodes, DiffusionEquation, LinearReactionDiffusionEquation, PoissonsEquation,
                  LaplacesEquation,
                  MeanExitTimeProblem, Tsit5, TRBDF2, KrylovSolver, SteadyFVMProblem, DynamicSS, NewtonRaphson,
                  SteadyStateSolution, ODESolution, LinearSolution, solve, BatchedProblem,
                  AdjointProblem, solve_rrule, FVMSystem, InvalidFluxError,
                  jacobian_sparsity, jvp, jacobian_diagonal, compute_flux, pl_interpolate, interpolate, two_point_interpolant,
                  construct_flux_function)
from ._lib import FVMError, UnsupportedFormError, NotConvergedError
from ._build import build, lib_path

__all__ = [
    "Triangulation", "triangulate_rectangle", "triangulate_annulus", "triangulate_disk", "triangulate_points",
    "ConditionType", "Neumann", "Dudt", "Dirichlet", "Constrained", "ParametrisedFunction", "BoundaryConditions",
    "InternalConditions", "Conditions", "TriangleProperties", "FVMGeometry", "FVMProblem", "fvm_eqs",
    "update_dirichlet_nodes", "DiffusionEquation", "LinearReactionDiffusionEquation", "PoissonsEquation",
    "MeanExitTimeProblem", "Tsit5", "KrylovSolver", "ODESolution", "LinearSolution", "solve", "BatchedProblem",
    "disjoint_union", "AdjointProblem", "solve_rrule", "FVMSystem", "InvalidFluxError", "jacobian_sparsity", "compute_flux", "pl_interpolate", "interpolate",
    "two_point_interpolant", "construct_flux_function", "FVMError",
    "UnsupportedFormError", "NotConvergedError", "build", "lib_path", "TRBDF2", "jvp", "jacobian_diagonal",
    "SteadyFVMProblem", "DynamicSS", "NewtonRaphson", "SteadyStateSolution", "LaplacesEquation",
]
