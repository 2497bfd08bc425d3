"""
    GridapHybridGB300

Julia binding of libgridaphybrid_gb300.so (C ABI: include/hdg_gb300.h) for
GridapHybrid.jl.  Loading it routes the reference's own calls to the GB300:

  - `lazy_map(StaticCondensationMap(bulk, skel), t)`, the call of
    src/HybridAffineFEOperators.jl:338, densifies every cell's (MatrixBlock,
    VectorBlock) once and condenses all cells in one `hdg_static_condensation`
    call; the result is a plain vector of `(S_c, g_c)` pairs, the same values
    the reference's map returns per cell (src/StaticCondensationMap.jl:146-196);
  - `lazy_map(BackwardStaticCondensationMap(bulk, skel), t, lhₖ)`, the call of
    src/HybridAffineFEOperators.jl:117-118, recovers all cells' interior DOFs in
    one `hdg_backward_static_condensation` call and re-blocks them as
    src/BackwardStaticCondensationMap.jl:133-151 does;
  - `HybridAffineFEOperator(form::DarcyHDGForm, X, Y, bulk, skel)` and
    `solve(op)` run the whole path (integrate, condense, assemble, skeleton
    solve, recover) on the GPU for the Darcy HDG form of
    test/DarcyHDGTests.jl:125-135, which is given as data (`DarcyHDGForm`),
    because a Gridap weak-form closure cannot cross the C ABI.  Gridap's own
    cell->facet and facet-DOF arrays are passed through `hdg_problem_create`,
    so the skeleton system is numbered exactly as Gridap numbers it.

Everything else of GridapHybrid is untouched.  There is no CPU fallback:
without a GB300, the first call raises.

Status: written against the C ABI and checked by the library's test-suite
(every `ccall`'s name, return type and argument types against the C
prototypes); not executed, because no Julia toolchain is available where this
library is built and tested.  The same entry points run from Python through
ctypes in the test-suite.
"""
module GridapHybridGB300

using Gridap
using Gridap.Arrays
using Gridap.Fields
using GridapHybrid
using LinearAlgebra

import Gridap.Arrays: lazy_map
import Gridap.FESpaces: solve
import GridapHybrid: StaticCondensationMap, BackwardStaticCondensationMap, HybridAffineFEOperator

const LIB = joinpath(@__DIR__, "..", "libgridaphybrid_gb300.so")

const HDG_OK = Cint(0)
const HDG_PREC_FP64 = Cint(0)
const HDG_PREC_FP32_REFINED = Cint(1)
const HDG_PREC_FF_BLOCK = Cint(2)      # float-float block elimination: the fastest operator path
const HDG_SOLVER_PCG = Cint(0)
const HDG_SOLVER_DIRECT = Cint(1)
const HDG_STAB_TEXTBOOK = Cint(0)
const HDG_STAB_OWNER_SIGN = Cint(1)

# Arithmetic of the Map-level calls (FP64 reproduces the reference's LAPACK
# sequence; FP32_REFINED is the FP32 LU with float-float refinement).
const MAP_PRECISION = Ref{Cint}(HDG_PREC_FP64)
set_map_precision!(p::Integer) = (MAP_PRECISION[] = Cint(p))

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
# Batched Map-level calls on densified cell blocks (column-major per cell).
# ---------------------------------------------------------------------------

# StaticCondensationMap over all cells (src/StaticCondensationMap.jl:146-196):
# A is n x n x ncells with the interior DOFs first, b is n x ncells.
function static_condensation!(S::Array{Float64,3}, g::Matrix{Float64}, info::Vector{Cint},
                              A::Array{Float64,3}, b::Matrix{Float64}, ni::Integer;
                              precision=MAP_PRECISION[], ctx=default_context())
  n, _, ncells = size(A)
  nf = n - ni
  check(ctx, ccall((:hdg_static_condensation, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                    Ptr{Float64}, Ptr{Cint}),
                   ctx.handle, precision, ncells, ni, nf, A, b, S, g, info))
  S, g
end

# BackwardStaticCondensationMap over all cells (src/BackwardStaticCondensationMap.jl:61-102):
# u[:, c] = A_ii^{-1} (b_i - A_if x[:, c]).
function backward_static_condensation!(u::Matrix{Float64}, info::Vector{Cint}, A::Array{Float64,3},
                                       b::Matrix{Float64}, x::Matrix{Float64}, ni::Integer;
                                       precision=HDG_PREC_FP64, ctx=default_context())
  n, _, ncells = size(A)
  nf = n - ni
  check(ctx, ccall((:hdg_backward_static_condensation, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                    Ptr{Float64}, Ptr{Cint}),
                   ctx.handle, precision, ncells, ni, nf, A, b, x, u, info))
  u
end

# Row sizes of a cell's field blocks (the reference's _compute_brs_bcs,
# src/StaticCondensationMap.jl:73-85).
function _field_sizes(A::MatrixBlock)
  brs = zeros(Int, size(A.array, 1))
  for j in 1:size(A.array, 2), i in 1:size(A.array, 1)
    A.touched[i, j] && (brs[i] = size(A.array[i, j], 1))
  end
  brs
end

# One cell's blocks, fields in `order` (interior fields first), densified into
# the column-major slices Ad (n x n) and bd (n); untouched blocks are zero
# (DensifyInnerMostBlockLevelMap's rule).
function _densify!(Ad, bd, A::MatrixBlock, b::VectorBlock, order, offs)
  fill!(Ad, 0.0)
  fill!(bd, 0.0)
  for (J, BJ) in enumerate(order), (I, BI) in enumerate(order)
    if A.touched[BI, BJ]
      blk = A.array[BI, BJ]
      Ad[offs[I]+1:offs[I]+size(blk, 1), offs[J]+1:offs[J]+size(blk, 2)] .= blk
    end
  end
  for (I, BI) in enumerate(order)
    if b.touched[BI]
      bd[offs[I]+1:offs[I]+length(b.array[BI])] .= b.array[BI]
    end
  end
end

# Densify every cell of a lazy cell array of (MatrixBlock, VectorBlock) pairs.
function _densify_cells(k::StaticCondensationMap, t::AbstractArray)
  ncells = length(t)
  cache = array_cache(t)
  A1, _ = getindex!(cache, t, 1)
  brs = _field_sizes(A1)
  order = vcat(k.interior_fields, k.boundary_fields)
  offs = cumsum(vcat(0, brs[order]))
  ni = sum(brs[k.interior_fields])
  n = offs[end]
  A = Array{Float64}(undef, n, n, ncells)
  b = Array{Float64}(undef, n, ncells)
  for c in 1:ncells
    Ac, bc = getindex!(cache, t, c)
    _densify!(view(A, :, :, c), view(b, :, c), Ac, bc, order, offs)
  end
  A, b, ni, brs
end

# lazy_map(StaticCondensationMap(bulk, skel), t) with t the skeleton matvec
# contribution (src/HybridAffineFEOperators.jl:333-341): every cell in one call.
function lazy_map(k::StaticCondensationMap, t::AbstractArray{<:Tuple{<:MatrixBlock,<:VectorBlock}})
  ncells = length(t)
  ncells == 0 && return Tuple{Matrix{Float64},Vector{Float64}}[]
  A, b, ni, _ = _densify_cells(k, t)
  n = size(A, 1)
  nf = n - ni
  S = Array{Float64}(undef, nf, nf, ncells)
  g = Array{Float64}(undef, nf, ncells)
  info = Vector{Cint}(undef, ncells)
  static_condensation!(S, g, info, A, b, ni)
  [(S[:, :, c], g[:, c]) for c in 1:ncells]
end

# The skeleton values of one cell as one dense vector (lhₖ may hold a
# VectorBlock per cell when the skeleton has several fields).
_dense(x::AbstractVector{<:Real}) = x
_dense(x::VectorBlock) = reduce(vcat, [x.array[i] for i in 1:length(x.array) if x.touched[i]])

# lazy_map(BackwardStaticCondensationMap(bulk, skel), t, lhₖ)
# (src/HybridAffineFEOperators.jl:115-118): every cell's interior recovered in
# one call, then re-blocked per field, interior blocks first and the skeleton
# blocks from lhₖ (ReblockInteriorDofsMap, src/BackwardStaticCondensationMap.jl:133-151).
function lazy_map(k::BackwardStaticCondensationMap, t::AbstractArray{<:Tuple{<:MatrixBlock,<:VectorBlock}},
                  lh::AbstractArray)
  sc = k.static_condensation
  ncells = length(t)
  ncells == 0 && return VectorBlock{Vector{Float64}}[]
  A, b, ni, brs = _densify_cells(sc, t)
  n = size(A, 1)
  nf = n - ni
  x = Matrix{Float64}(undef, nf, ncells)
  xcache = array_cache(lh)
  for c in 1:ncells
    x[:, c] .= _dense(getindex!(xcache, lh, c))
  end
  u = Matrix{Float64}(undef, ni, ncells)
  info = Vector{Cint}(undef, ncells)
  backward_static_condensation!(u, info, A, b, x, ni)
  ibrs = brs[sc.interior_fields]
  bbrs = brs[sc.boundary_fields]
  map(1:ncells) do c
    blocks = Vector{Vector{Float64}}(undef, length(ibrs) + length(bbrs))
    o = 0
    for (i, s) in enumerate(ibrs)
      blocks[i] = u[o+1:o+s, c]
      o += s
    end
    o = 0
    for (i, s) in enumerate(bbrs)
      blocks[length(ibrs)+i] = x[o+1:o+s, c]
      o += s
    end
    ArrayBlock(blocks, fill(true, length(blocks)))
  end
end

# ---------------------------------------------------------------------------
# HybridAffineFEOperator + solve on the GPU for the Darcy HDG form.
# ---------------------------------------------------------------------------

"""
    DarcyHDGForm(order; tau=1.0, stabilization=:owner_sign, kappa=nothing, problem=0)

The Darcy HDG weak form of test/DarcyHDGTests.jl:125-135 as data: flux and
pressure Q_order inside the cells, a facet multiplier of the same order,
stabilisation `τ(p−l)(n⋅nₒ)` (`:owner_sign`, the reference's) or `τ(p−l)`
(`:textbook`), an optional per-cell permeability in the flux mass term and one
of the library's manufactured problems (HDG_PROBLEM_*) for the source and the
Dirichlet data.
"""
struct DarcyHDGForm
  order::Int
  tau::Float64
  stabilization::Symbol
  kappa::Union{Nothing,Vector{Float64}}
  problem::Cint
end
DarcyHDGForm(order::Integer; tau=1.0, stabilization=:owner_sign, kappa=nothing, problem=0) =
  DarcyHDGForm(order, tau, stabilization, kappa, Cint(problem))

mutable struct GPUHybridOperator
  ctx::Context
  problem::Ptr{Cvoid}
  trial::Any
  test::Any
  D::Int
  ncells::Int
  ni::Int
  nfree::Int
  precision::Cint
end

function _destroy!(op::GPUHybridOperator)
  if op.problem != C_NULL
    ccall((:hdg_problem_destroy, LIB), Cint, (Ptr{Cvoid},), op.problem)
    op.problem = C_NULL
  end
end

# Gridap's own numbering, passed through hdg_problem_create: cell->facets
# (get_faces(topo, D, D-1), src/HybridAffineFEOperators.jl:152-156), the
# affine cell maps, and the facet space's DOF ids (get_cell_dof_ids(M), with
# Gridap's sign convention for Dirichlet DOFs).
function GPUHybridOperator(model::DiscreteModel, order::Integer, M; precision=HDG_PREC_FF_BLOCK,
                           ctx=default_context(), trial=nothing, test=nothing)
  D = num_cell_dims(model)
  topo = get_grid_topology(model)
  cell_facets = Gridap.Geometry.get_faces(topo, D, D - 1)
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
  info = Vector{Clonglong}(undef, 8)
  check(ctx, ccall((:hdg_problem_info, LIB), Cint, (Ptr{Cvoid}, Ptr{Clonglong}), h[], info))
  op = GPUHybridOperator(ctx, h[], trial, test, D, info[1], info[3], info[5], Cint(precision))
  finalizer(_destroy!, op)
  op
end

function set_form!(op::GPUHybridOperator, form::DarcyHDGForm)
  stab = form.stabilization == :owner_sign ? HDG_STAB_OWNER_SIGN : HDG_STAB_TEXTBOOK
  check(op.ctx, ccall((:hdg_set_darcy, LIB), Cint, (Ptr{Cvoid}, Cint, Cdouble, Cint),
                      op.problem, stab, form.tau, form.problem))
  kp = form.kappa === nothing ? Ptr{Float64}(C_NULL) : pointer(form.kappa)
  GC.@preserve form check(op.ctx, ccall((:hdg_set_permeability, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}),
                                        op.problem, kp))
  op
end

"""
    HybridAffineFEOperator(form::DarcyHDGForm, X, Y, bulk_fields, skeleton_fields; precision)

The GPU counterpart of `HybridAffineFEOperator(weakform, X, Y, bulk, skel)`
(src/HybridAffineFEOperators.jl:10-50) for the Darcy HDG form: integrates,
condenses and assembles the skeleton system on the GPU, with the numbering of
the skeleton space `X[skeleton_fields[1]]`.  `solve(op)` then solves and
recovers, as `solve(op::HybridAffineFEOperator)` does (:67-100).
"""
function HybridAffineFEOperator(form::DarcyHDGForm, trial::MultiFieldFESpace, test::MultiFieldFESpace,
                                bulk_fields::Vector{<:Integer}, skeleton_fields::Vector{<:Integer};
                                precision=HDG_PREC_FF_BLOCK, ctx=default_context())
  length(skeleton_fields) == 1 || error("the GPU Darcy operator has one skeleton field")
  M = trial[skeleton_fields[1]]
  model = get_background_model(get_triangulation(trial[bulk_fields[1]]))
  op = GPUHybridOperator(model, form.order, M; precision=precision, ctx=ctx, trial=trial, test=test)
  set_form!(op, form)
  check(op.ctx, ccall((:hdg_assemble, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Cint}), op.problem, op.precision,
                      Ptr{Cint}(C_NULL)))
  op
end

"""
    solve(op::GPUHybridOperator; solver, rtol, maxit)

Skeleton solve, interior recovery and the free DOF values in Gridap's layout
[flux | pressure | skeleton] (src/HybridAffineFEOperators.jl:72-100); returns
`FEFunction(op.trial, free_dof_values)` when the operator was built from
Gridap spaces, else the free DOF values.
"""
function solve(op::GPUHybridOperator; solver=HDG_SOLVER_PCG, rtol=1e-10, maxit=20000)
  its = Ref{Cint}(0)
  rel = Ref{Cdouble}(0)
  check(op.ctx, ccall((:hdg_solve_skeleton, LIB), Cint,
                      (Ptr{Cvoid}, Cint, Cdouble, Cint, Ptr{Cint}, Ptr{Cdouble}),
                      op.problem, solver, rtol, maxit, its, rel))
  check(op.ctx, ccall((:hdg_recover, LIB), Cint, (Ptr{Cvoid},), op.problem))
  free = Vector{Float64}(undef, op.ncells * op.ni + op.nfree)
  check(op.ctx, ccall((:hdg_get_free_dof_values, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), op.problem, free))
  op.trial === nothing ? free : FEFunction(op.trial, free)
end

# solve(op) in one call with a new permeability field (src/HybridAffineFEOperators.jl:67-100):
# sets kappa (one value per cell), assembles in `precision`, solves the skeleton, recovers
# and returns the free DOF values; `stats` = [iterations, relative residual, ms integrate +
# condense, ms assemble, ms solve, ms recover, ms total].
function solve!(op::GPUHybridOperator, kappa::Vector{Float64}; precision=op.precision,
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

const HDG_PHYSICS_DARCY = Cint(0)
const _SPACE_KIND = Dict(:Q => Cint(0), :P => Cint(1), :RT => Cint(2))

"""
    HybridAffineFEOperator(form::DarcyHDGForm, model::CartesianDiscreteModel, spaces;
                           copies=1, precision=HDG_PREC_FP64)

The Darcy HDG form on a Cartesian model with a space per field, as the
reference's tests declare them: `spaces = (kindA, kA, kindB, kB, kindT, kT)`
with kinds `:Q` (`space=:Q`), `:P` (`space=:P`) or, for the flux, `:RT`
(`ReferenceFE(raviart_thomas, Float64, k)`): `(:P, 1, :P, 0, :P, 1)` is
test/DarcyHDGTests.jl:34-36, `(:RT, 0, :Q, 0, :Q, 0)` with `tau = 0` the RT-H
form of test/DarcyRTHTests.jl:65-72.  `copies = c` builds the multi-field
space [U_1..U_c, P_1..P_c, L_1..L_c] with bulk fields 1:2c and skeleton fields
2c+1:3c, the block form repeated per copy
(test/MultiFieldLagrangeMultipliersTests.jl:40-88); the free DOF values come
back in that multi-field order.  Condensation in FP64 or FP32 with float-float
refinement (`HDG_PREC_FF_BLOCK` needs equal-order Q_k fields).  With
`simplexified = true` the model is simplexified first (2 triangles per square,
6 tetrahedra per cube) and the fields must be `:P`.
"""
function HybridAffineFEOperator(form::DarcyHDGForm, model::CartesianDiscreteModel, spaces::Tuple;
                                copies::Integer=1, precision=HDG_PREC_FP64, ctx=default_context(),
                                trial=nothing, test=nothing, simplexified::Bool=false)
  desc = get_cartesian_descriptor(model)
  D = length(desc.partition)
  cells = Cint[desc.partition...]
  domain = Float64[]
  for d in 1:D
    push!(domain, desc.origin[d], desc.origin[d] + desc.sizes[d] * desc.partition[d])
  end
  sp = Cint[_SPACE_KIND[spaces[1]], spaces[2], _SPACE_KIND[spaces[3]], spaces[4], _SPACE_KIND[spaces[5]],
            spaces[6], 0]
  h = Ref{Ptr{Cvoid}}(C_NULL)
  if simplexified
    # simplexify(model) with the library's own split and numbering (test/DarcyHDGTests.jl:174-177)
    check(ctx, ccall((:hdg_problem_create_simplex_spaces, LIB), Cint,
                     (Ptr{Cvoid}, Cint, Ptr{Cint}, Ptr{Float64}, Cint, Ptr{Cint}, Cint, Ptr{Ptr{Cvoid}}),
                     ctx.handle, D, cells, domain, HDG_PHYSICS_DARCY, sp, copies, h))
  else
    check(ctx, ccall((:hdg_problem_create_cartesian_spaces, LIB), Cint,
                     (Ptr{Cvoid}, Cint, Ptr{Cint}, Ptr{Float64}, Cint, Ptr{Cint}, Cint, Ptr{Ptr{Cvoid}}),
                     ctx.handle, D, cells, domain, HDG_PHYSICS_DARCY, sp, copies, h))
  end
  info = Vector{Clonglong}(undef, 8)
  check(ctx, ccall((:hdg_problem_info, LIB), Cint, (Ptr{Cvoid}, Ptr{Clonglong}), h[], info))
  op = GPUHybridOperator(ctx, h[], trial, test, D, info[1], info[3], info[5], Cint(precision))
  finalizer(_destroy!, op)
  set_form!(op, form)
  check(op.ctx, ccall((:hdg_assemble, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Cint}), op.problem, op.precision,
                      Ptr{Cint}(C_NULL)))
  op
end

export DarcyHDGForm, GPUHybridOperator, l2_errors, set_refinement!, set_map_precision!

end # module
