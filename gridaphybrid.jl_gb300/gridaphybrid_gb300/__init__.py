"""gridaphybrid_gb300 -- GridapHybrid.jl's cellwise hybridization hot path on a
GB300 (sm_103a), behind the reference's Map / HybridAffineFEOperator / solve API.

The numerics live in libgridaphybrid_gb300.so (C ABI: include/hdg_gb300.h);
this package is the host-side mirror of the reference interface.
"""
from . import _lib
from ._lib import Context, HdgError, default_context
from .maps import (ArrayBlock, BackwardStaticCondensationMap, MatrixBlock,
                   Scalar2ArrayBlockMap, StaticCondensationMap, SumFacetsMap, VectorBlock,
                   densify, evaluate, lazy_map, return_cache)
from .operators import (CartesianDiscreteModel, DarcyHDG, ElasticityHDG, FEFunction, FESolver,
                        HybridAffineFEOperator, HybridFEOperator, MultiFieldFESpace,
                        NLSolver, ReferenceFE, Skeleton, TestFESpace, TrialFESpace,
                        Triangulation, darcy_spaces, elasticity_spaces, get_cell_normal_vector,
                        get_cell_owner_normal_vector, lagrangian, raviart_thomas, simplexify, solve,
                        solve_)

__all__ = [
    "ArrayBlock", "BackwardStaticCondensationMap", "CartesianDiscreteModel", "Context",
    "DarcyHDG", "ElasticityHDG", "FEFunction", "FESolver", "HdgError", "HybridAffineFEOperator", "HybridFEOperator",
    "NLSolver", "MatrixBlock", "MultiFieldFESpace",
    "ReferenceFE", "Scalar2ArrayBlockMap", "Skeleton", "StaticCondensationMap", "SumFacetsMap", "TestFESpace",
    "TrialFESpace", "Triangulation", "VectorBlock", "darcy_spaces", "default_context",
    "densify", "elasticity_spaces", "evaluate", "get_cell_normal_vector", "get_cell_owner_normal_vector",
    "lagrangian", "lazy_map", "raviart_thomas", "return_cache", "simplexify", "solve", "solve_",
]
