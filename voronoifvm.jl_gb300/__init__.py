"""GB300-native assembly + Newton hot path of VoronoiFVM.jl.

The compute path is the CUDA library built from ``csrc/`` (C ABI in
``include/vfvm_gb300.h``); this package is its host-side mirror of the
reference's ``System``/``Physics``/``solve``/``SolverControl`` interface.
"""
from .grid import Grid, bfacemask, cellmask, circular_symmetric, read_sg, simplexgrid, spherical_symmetric, write_sg
from .system import (AssemblyError, ConvergenceError, EmbeddingError, LinearSolverError, NewtonSolverHistory,
                     Physics, SolverControl, System, TransientSolution, boundary_dirichlet, edgefactors,
                     enable_boundary_species, enable_species, evaluate_residual_and_jacobian, fixed_timesteps,
                     integrate, integrate_gradT_flux, node_species, nodevolumes, num_species, solve,
                     TestFunctionFactory, testfunction, unknowns, eval_rhs, eval_jacobian, mass_matrix,
                     parameter_derivatives)
from . import _lib
from .batch import BatchSolver
from . import learned
from .build import build_library

__all__ = ["Grid", "simplexgrid", "cellmask", "bfacemask", "circular_symmetric", "spherical_symmetric", "read_sg", "write_sg",
           "Physics", "System", "SolverControl", "NewtonSolverHistory", "TransientSolution",
           "AssemblyError", "ConvergenceError", "EmbeddingError", "LinearSolverError", "boundary_dirichlet",
           "enable_species", "enable_boundary_species", "node_species", "TestFunctionFactory", "testfunction",
           "integrate_gradT_flux", "eval_rhs", "eval_jacobian", "mass_matrix", "parameter_derivatives",
           "edgefactors", "evaluate_residual_and_jacobian", "fixed_timesteps", "integrate", "nodevolumes",
           "num_species", "solve", "unknowns", "build_library"]
