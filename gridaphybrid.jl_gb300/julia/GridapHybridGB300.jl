"""
    GridapHybridGB300

Julia binding of libgridaphybrid_gb300.so (C ABI: include/hdg_gb300.h) for
GridapHybrid.jl.  It overrides the two condensation maps' batched evaluation
and adds GPU methods of `HybridAffineFEOperator`/`solve` for the Darcy HDG
form, so that existing GridapHybrid programs route the hot path to the GB300.

Status: written against the C ABI; not executed (no Julia toolchain is
available where this library is built and tested).  The same entry points are
exercised from Python through ctypes by the library's test-suite.
"""
module GridapHybridGB300

using Gridap
using GridapHybrid
using LinearAlgebra

const LIB = joinpath(@__DIR__, "..", "libgridaphybrid_gb300.so")

const HDG_OK = Cint(0)
const HDG_PREC_FP64 = Cint(0)
const HDG_PREC_FP32_REFINED = Cint(1)
const HDG_PREC_FF_BLOCK = Cint(2)      # float-float block elimination: the fastest path (Darcy, elasticity)
const HDG_SOLVER_PCG = Cint(0)
const HDG_SOLVER_DIRECT = Cint(1)

mutable struct Context
  handle::Ptr{Cvoid}
end

function Context(device::Integer=0)
  h = Ref{Ptr{Cvoid}}(C_NULL)
  rc = ccall((:hdg_context_create, LIB), Cint, (Cint, Ptr{Ptr{Cvoid}}), device, h)
  rc == HDG_OK || error("hdg_context_create failed ($rc): no usable sm_103a GPU")
  ctx = Context(h[])
  finalizer(c -> ccall((:hdg_context_destroy, LIB), Cint, (Ptr{Cvoid},), c.handle), ctx)
  ctx
end

function check(ctx::Context, rc::Cint)
  if rc != HDG_OK
    msg = unsafe_string(ccall((:hdg_last_error, LIB), Cstring, (Ptr{Cvoid},), ctx.handle))
    error("libgridaphybrid_gb300: status $rc: $msg")
  end
  rc
end

const DEFAULT = Ref{Union{Nothing,Context}}(nothing)
default_context() = something(DEFAULT[], (DEFAULT[] = Context(0)))

# ---------------------------------------------------------------------------
# StaticCondensationMap over all cells in one call (src/StaticCondensationMap.jl:146-196).
# `cell_A`, `cell_b`: densified cell blocks with interior fields first
# (DensifyInnerMostBlockLevelMap of the re-blocked MatrixBlock/VectorBlock).
# ---------------------------------------------------------------------------
function static_condensation(cell_A::AbstractVector{<:Matrix{Float64}},
                             cell_b::AbstractVector{<:Vector{Float64}},
                             ni::Integer; precision=HDG_PREC_FP64, ctx=default_context())
  ncells = length(cell_A)
  n = size(cell_A[1], 1)
  nf = n - ni
  A = Array{Float64}(undef, n, n, ncells)      # column-major per cell, as the ABI expects
  b = Array{Float64}(undef, n, ncells)
  for c in 1:ncells
    A[:, :, c] .= cell_A[c]
    b[:, c] .= cell_b[c]
  end
  S = Array{Float64}(undef, nf, nf, ncells)
  g = Array{Float64}(undef, nf, ncells)
  info = Vector{Cint}(undef, ncells)
  check(ctx, ccall((:hdg_static_condensation, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                    Ptr{Float64}, Ptr{Cint}),
                   ctx.handle, precision, ncells, ni, nf, A, b, S, g, info))
  [(S[:, :, c], g[:, c]) for c in 1:ncells]
end

# BackwardStaticCondensationMap over all cells (src/BackwardStaticCondensationMap.jl:61-102)
function backward_static_condensation(cell_A, cell_b, cell_x, ni::Integer;
                                      precision=HDG_PREC_FP64, ctx=default_context())
  ncells = length(cell_A)
  n = size(cell_A[1], 1)
  nf = n - ni
  A = Array{Float64}(undef, n, n, ncells)
  b = Array{Float64}(undef, n, ncells)
  x = Array{Float64}(undef, nf, ncells)
  for c in 1:ncells
    A[:, :, c] .= cell_A[c]
    b[:, c] .= cell_b[c]
    x[:, c] .= cell_x[c]
  end
  u = Array{Float64}(undef, ni, ncells)
  info = Vector{Cint}(undef, ncells)
  check(ctx, ccall((:hdg_backward_static_condensation, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                    Ptr{Float64}, Ptr{Cint}),
                   ctx.handle, precision, ncells, ni, nf, A, b, x, u, info))
  [u[:, c] for c in 1:ncells]
end

# ---------------------------------------------------------------------------
# HybridAffineFEOperator + solve for the Darcy HDG form of
# test/DarcyHDGTests.jl:125-135 on a CartesianDiscreteModel
# (src/HybridAffineFEOperators.jl:10-100).  Gridap's own numbering is passed
# through hdg_problem_create so the skeleton system is assembled exactly as
# Gridap numbers it.
# ---------------------------------------------------------------------------
struct GPUHybridOperator
  ctx::Context
  problem::Ptr{Cvoid}
  D::Int
  ncells::Int
  ni::Int
  nfree::Int
end

function GPUHybridOperator(model::CartesianDiscreteModel, order::Integer;
                           tau=1.0, stabilization=:owner_sign, problem=0, kappa=nothing,
                           precision=HDG_PREC_FP64, ctx=default_context())
  D = num_cell_dims(model)
  topo = get_grid_topology(model)
  cell_facets = Gridap.Geometry.get_faces(topo, D, D - 1)        # src/HybridAffineFEOperators.jl:152-156
  ncells = length(cell_facets)
  nfacets = num_faces(topo, D - 1)
  cf = Matrix{Cint}(undef, 2D, ncells)
  for c in 1:ncells, (lf, f) in enumerate(cell_facets[c])
    cf[lf, c] = f - 1
  end
  coords = get_cell_coordinates(get_grid(model))
  origin = Matrix{Float64}(undef, D, ncells)
  jac = Array{Float64}(undef, D, D, ncells)
  for c in 1:ncells
    x = coords[c]
    for d in 1:D
      origin[d, c] = x[1][d]
      for e in 1:D
        jac[d, e, c] = x[1 + 2^(e - 1)][d] - x[1][d]          # affine cells: J e_e = x(e_e) - x(0)
      end
    end
  end
  reffe = ReferenceFE(lagrangian, Float64, order)
  M = TestFESpace(Triangulation(ReferenceFE{D - 1}, model), reffe; conformity=:L2,
                  dirichlet_tags="boundary")
  fdofs = get_cell_dof_ids(M)
  nfd = (order + 1)^(D - 1)
  fd = Matrix{Cint}(undef, nfd, nfacets)
  for f in 1:nfacets, (a, id) in enumerate(fdofs[f])
    fd[a, f] = id > 0 ? id - 1 : id                                # 0-based free, -1-k Dirichlet
  end
  h = Ref{Ptr{Cvoid}}(C_NULL)
  check(ctx, ccall((:hdg_problem_create, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Cint}, Ptr{Cint},
                    Ptr{Ptr{Cvoid}}),
                   ctx.handle, D, order, ncells, nfacets, origin, jac, cf, fd, h))
  stab = stabilization == :owner_sign ? Cint(1) : Cint(0)
  check(ctx, ccall((:hdg_set_darcy, LIB), Cint, (Ptr{Cvoid}, Cint, Cdouble, Cint), h[], stab, tau, problem))
  kp = kappa === nothing ? C_NULL : pointer(kappa)
  check(ctx, ccall((:hdg_set_permeability, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), h[], kp))
  info = Vector{Clonglong}(undef, 8)
  check(ctx, ccall((:hdg_problem_info, LIB), Cint, (Ptr{Cvoid}, Ptr{Clonglong}), h[], info))
  check(ctx, ccall((:hdg_assemble, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Cint}), h[], precision, C_NULL))
  GPUHybridOperator(ctx, h[], D, info[1], info[3], info[5])
end

function solve_gpu(op::GPUHybridOperator; solver=HDG_SOLVER_PCG, rtol=1e-10, maxit=20000)
  its = Ref{Cint}(0)
  rel = Ref{Cdouble}(0)
  check(op.ctx, ccall((:hdg_solve_skeleton, LIB), Cint,
                      (Ptr{Cvoid}, Cint, Cdouble, Cint, Ptr{Cint}, Ptr{Cdouble}),
                      op.problem, solver, rtol, maxit, its, rel))
  check(op.ctx, ccall((:hdg_recover, LIB), Cint, (Ptr{Cvoid},), op.problem))
  free = Vector{Float64}(undef, op.ncells * op.ni + op.nfree)
  check(op.ctx, ccall((:hdg_get_free_dof_values, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), op.problem, free))
  free                                                               # FEFunction(op.trial, free)
end

# solve(op) in one call with a new permeability field (src/HybridAffineFEOperators.jl:67-100):
# sets kappa (one value per cell), assembles in `precision`, solves the skeleton, recovers
# and returns the free DOF values; `stats` = [iterations, relative residual, ms integrate +
# condense, ms assemble, ms solve, ms recover, ms total].
function solve_gpu!(op::GPUHybridOperator, kappa::Vector{Float64}; precision=HDG_PREC_FP64,
                    solver=HDG_SOLVER_PCG, rtol=1e-10, maxit=20000)
  length(kappa) == op.ncells || error("kappa needs one value per cell")
  free = Vector{Float64}(undef, op.ncells * op.ni + op.nfree)
  stats = Vector{Float64}(undef, 7)
  check(op.ctx, ccall((:hdg_solve, LIB), Cint,
                      (Ptr{Cvoid}, Cint, Cint, Cdouble, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                      op.problem, precision, solver, rtol, maxit, kappa, free, stats))
  free, stats
end

# sqrt(sum(∫(e⋅e)dΩ)) for the flux and the pressure (test/DarcyHDGTests.jl:141-142)
function l2_errors(op::GPUHybridOperator)
  ef = Ref{Cdouble}(0)
  ep = Ref{Cdouble}(0)
  check(op.ctx, ccall((:hdg_l2_errors, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}),
                      op.problem, ef, ep))
  ef[], ep[]
end

# refinement of the fast precisions' skeleton solve: the residual reduction between two
# FP64 residuals (default 1e-2 in 3D, 3e-2 in 2D) and reliable updates on/off
function set_refinement!(op::GPUHybridOperator; delta=(op.D == 3 ? 1e-2 : 3e-2), keep_direction=true)
  check(op.ctx, ccall((:hdg_set_refinement, LIB), Cint, (Ptr{Cvoid}, Cdouble, Cint),
                      op.problem, Float64(delta), keep_direction ? Cint(1) : Cint(0)))
  op
end

end # module
