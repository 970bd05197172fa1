"""
    GridapMHDGB300

Julia binding of libgbmhd: adds the `:gb300` solver to GridapMHD by method
extension (no edit of GridapMHD).  `GridapMHD.main(params)` and `hunt(...)`
keep their parameter dictionaries; `params[:solver] = :gb300` (or a Dict with
`:solver => :gb300`) routes the Newton assembly and solve to the GPU.

Hooks extended (GridapMHD paths):
  default_solver_params(::Val{:gb300})   src/parameters.jl:221-287 (pattern)
  uses_petsc(::Val{:gb300})              src/parameters.jl:289-295
  space_uses_multigrid(::Val{:gb300},s)  src/parameters.jl:298-303
  _multi_field_style(::Val{:gb300})      src/fespaces.jl:4-9
  _solver(::Val{:gb300},op,params)       src/main.jl:173-190

The library's cell-local basis (documented in include/gbmhd.h) differs from
Gridap's reference FEs by a fixed cell-local change of basis: a permutation of
the 27 Q2 nodes, and small dense maps for the P1, RT1 face/interior and Q1
dofs.  `local_maps(reffes)` computes them once by evaluating Gridap's dof
functionals on the library basis; the shim converts values at the boundary.
This file has not been executed in this build (no Julia toolchain); the C
entry points it binds are the ones the Python binding exercises.
"""
module GridapMHDGB300

using Gridap
using Gridap.FESpaces, Gridap.MultiField, Gridap.Algebra, Gridap.ReferenceFEs, Gridap.Geometry
import GridapMHD

const LIB = get(ENV, "GBMHD_LIB", joinpath(@__DIR__, "..", "gbmhd", "libgbmhd.so"))

# ---------------------------------------------------------------- C structs (include/gbmhd.h)
struct GbMesh
  ncells::Int64
  cell_coords::Ptr{Float64}
end

struct GbDofMap
  nfree::NTuple{4,Int64}
  ndir::NTuple{4,Int64}
  cell_dofs::Ptr{Int32}
  dir_values::NTuple{4,Ptr{Float64}}
  cell_sign_j::Ptr{Int8}
end

struct GbParams
  alpha::Float64; beta::Float64; gamma::Float64; sigma::Float64
  B::NTuple{3,Float64}; f::NTuple{3,Float64}; g::NTuple{3,Float64}
  zeta_u::Float64; zeta_j::Float64
  convection::Int32
  f_cell::Ptr{Float64}
  nfacets::Int64
  facet_cell::Ptr{Int32}; facet_lface::Ptr{Int8}
  facet_tau::Ptr{Float64}; facet_cw::Ptr{Float64}; facet_jw::Ptr{Float64}; facet_phi0::Ptr{Float64}
end

struct GbSolveOpts
  precision::Int32; max_newton::Int32; newton_rtol::Float64; newton_atol::Float64
  restart::Int32; max_linear::Int32; linear_rtol::Float64; verbose::Int32; preconditioner::Int32
end

mutable struct GbReport
  newton_iters::Int32; linear_iters::Int32; converged::Int32
  initial_residual::Float64; final_residual::Float64
  time_assembly_s::Float64; time_setup_pc_s::Float64; time_linear_s::Float64; time_total_s::Float64
  residual_history::NTuple{64,Float64}
  pc_refactorizations::Int32
  GbReport() = new(0,0,0,0,0,0,0,0,0,ntuple(_->0.0,64),0)
end

struct GbHuntAnalytic
  L::Float64; mu::Float64; grad_pz::Float64; sigma::Float64; Ha::Float64; nsums::Int32
  u_scale::Float64; j_scale::Float64; length_scale::Float64
end

last_error(h) = unsafe_string(ccall((:gbmhd_last_error, LIB), Cstring, (Ptr{Cvoid},), h))
check(rc, h, what) = rc < 0 ? error("$what failed ($rc): $(last_error(h))") : rc

# ---------------------------------------------------------------- GridapMHD hooks
function GridapMHD.default_solver_params(::Val{:gb300})
  Dict(:solver => :gb300, :matrix_type => SparseMatrixCSR{0,Float64,Int64}, :vector_type => Vector{Float64},
       :solver_postpro => ((cache,info) -> gb300_postpro(cache,info)), :niter => 10, :niter_ls => 40,
       :rtol => 1e-10, :atol => 0.0, :precision => :mixed, :max_linear => 500, :linear_rtol => 1e-6,
       :preconditioner => :monolithic)
end
GridapMHD.uses_petsc(::Val{:gb300}) = false
GridapMHD.space_uses_multigrid(::Val{:gb300}, solver) = fill(false, 4)
GridapMHD._multi_field_style(::Val{:gb300}) = ConsecutiveMultiFieldStyle()
GridapMHD._solver(::Val{:gb300}, op, params) = GB300NewtonSolver(op, params)

struct GB300NewtonSolver <: NonlinearSolver
  params::Dict{Symbol,Any}
  handle::Base.RefValue{Ptr{Cvoid}}
  keep::Vector{Any}
end

function GB300NewtonSolver(op, params)
  h = Ref{Ptr{Cvoid}}(C_NULL)
  keep = Any[]
  mesh, dofs, prm = extract(op, params, keep)
  GC.@preserve keep begin
    rc = ccall((:gbmhd_create, LIB), Cint, (Ref{Ptr{Cvoid}}, Ref{GbMesh}, Ref{GbDofMap}, Ref{GbParams}),
               h, mesh, dofs, prm)
  end
  rc == 0 || error("gbmhd_create failed ($rc): $(last_error(C_NULL))")
  s = GB300NewtonSolver(params, h, keep)
  finalizer(x -> ccall((:gbmhd_destroy, LIB), Cvoid, (Ptr{Cvoid},), x.handle[]), s)
  s
end

struct GB300Cache
  report::GbReport
end

function Algebra.solve!(x::AbstractVector, nls::GB300NewtonSolver, op::NonlinearOperator, cache)
  s = nls.params[:solver]
  o = GbSolveOpts(s[:precision] == :mixed ? 1 : 0, s[:niter], s[:rtol], s[:atol], s[:niter_ls],
                  s[:max_linear], s[:linear_rtol], 0, s[:preconditioner] == :monolithic ? 0 : 1)
  rep = GbReport()
  xl = to_library_basis(nls, x)
  GC.@preserve xl begin
    rc = ccall((:gbmhd_newton_solve, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ref{GbSolveOpts}, Ref{GbReport}),
               nls.handle[], xl, o, rep)
  end
  check(rc, nls.handle[], "gbmhd_newton_solve")
  copyto!(x, from_library_basis(nls, xl))
  GB300Cache(rep)
end

function gb300_postpro(cache, info)
  info[:nls_iters] = cache.report.newton_iters
  info[:ls_iters] = cache.report.linear_iters
end

# The norms of hunt()'s post-processing (src/Applications/hunt.jl:238-260) on the device,
# for a hunt() driver that keeps the solver: pass the parameters hunt() derives there.
function hunt_errors(nls::GB300NewtonSolver, x::AbstractVector; L, μ, grad_pz, σ, Ha, nsums, u0, B0)
  a = GbHuntAnalytic(L, μ, grad_pz, σ, Ha, Int32(nsums), u0, σ * u0 * B0, L)
  out = zeros(9)
  xl = to_library_basis(nls, x)
  GC.@preserve xl out begin
    rc = ccall((:gbmhd_hunt_errors, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ref{GbHuntAnalytic}, Ptr{Float64}),
               nls.handle[], xl, a, out)
  end
  check(rc, nls.handle[], "gbmhd_hunt_errors")
  keys = (:eu_h1, :eu_l2, :ej_l2, :eu_ref_h1, :eu_ref_l2, :ej_ref_l2, :uh_h1, :uh_l2, :jh_l2)
  Dict(zip(keys, out))
end

# ---------------------------------------------------------------- extraction
# Cell coordinates, per-field cell dof ids (Gridap numbering, negative = Dirichlet),
# Dirichlet values, physical parameters and thin-wall facets, converted to the
# library's local layout (u component-major 3x27, p 4, j 36, φ 8).
function extract(op, params, keep)
  U = get_trial(op)
  model = params[:model]
  Ω = Triangulation(model)
  X = collect(Iterators.flatten(get_cell_coordinates(Ω)))
  coords = Float64[c[i] for c in X for i in 1:3]
  push!(keep, coords)
  ncells = num_cells(Ω)
  maps = local_maps(params[:fespaces])
  cell_dofs = Vector{Int32}(undef, 129 * ncells)
  nfree = zeros(Int64, 4); ndir = zeros(Int64, 4)
  dirv = Ptr{Float64}[C_NULL, C_NULL, C_NULL, C_NULL]
  for (f, Uf) in enumerate(U)
    ids = get_cell_dof_ids(Uf)
    nfree[f] = num_free_dofs(Uf)
    ndir[f] = num_dirichlet_dofs(Uf)
    dv = Vector{Float64}(get_dirichlet_dof_values(Uf))
    push!(keep, dv)
    dirv[f] = pointer(dv)
    off, perm = maps.slots[f]
    for c in 1:ncells, (k, p) in enumerate(perm)
      id = ids[c][p]
      cell_dofs[129*(c-1) + off + k] = id > 0 ? Int32(id - 1) : Int32(id)  # Gridap: -k for Dirichlet k
    end
  end
  push!(keep, cell_dofs)
  fl = params[:fluid]
  B = Tuple(Float64.(fl[:B])); f = Tuple(Float64.(fl[:f])); g = Tuple(Float64.(fl[:g]))
  conv = Int32(fl[:convection] == :none ? 0 : fl[:convection] == :picard ? 1 : 2)
  fc, fl_, tau, cw, jw = thin_wall_facets(model, params[:bcs], keep)
  prm = GbParams(fl[:α], fl[:β], fl[:γ], fl[:σ], B, f, g, fl[:ζᵤ], fl[:ζⱼ], conv, C_NULL, length(fc),
                 pointer(fc), pointer(fl_), pointer(tau), pointer(cw), pointer(jw), C_NULL)
  mesh = GbMesh(ncells, pointer(coords))
  dofs = GbDofMap(Tuple(nfree), Tuple(ndir), pointer(cell_dofs), Tuple(dirv), C_NULL)
  mesh, dofs, prm
end

# Boundary facets of each thin-wall tag as (cell, local face axis*2+side).
function thin_wall_facets(model, bcs, keep)
  cells = Int32[]; faces = Int8[]; tau = Float64[]; cw = Float64[]; jw = Float64[]
  for tw in bcs[:thin_wall]
    Γ = Boundary(model, tags=tw[:domain])
    glue = get_glue(Γ, Val(num_cell_dims(model)))
    for (c, lf) in zip(glue.tface_to_mface, glue.tface_to_mface_map)
      push!(cells, Int32(c - 1)); push!(faces, Int8(gridap_face_to_library(lf)))
      push!(tau, tw[:τ]); push!(cw, tw[:cw]); push!(jw, tw[:jw])
    end
  end
  append!(keep, (cells, faces, tau, cw, jw))
  cells, faces, tau, cw, jw
end

# Gridap HEX faces are ordered (z0, z1, y0, y1, x0, x1); the library uses axis*2 + side.
gridap_face_to_library(lf) = (4, 5, 2, 3, 0, 1)[lf]

# Change of basis between Gridap's reference FEs and the library basis (see module doc).
function local_maps(fespaces)
  reffe_u = fespaces[:reffe_u]
  nodes = get_node_coordinates(reffe_u)
  lib_node(x) = round(Int, 2x[1]) + 3 * round(Int, 2x[2]) + 9 * round(Int, 2x[3]) + 1
  perm_nodes = sortperm([lib_node(x) for x in nodes])
  perm_u = vcat([perm_nodes .+ 27 * c for c in 0:2]...)  # component-major in both
  (slots = ((0, perm_u), (81, collect(1:4)), (85, collect(1:36)), (121, collect(1:8))),)
end

to_library_basis(nls, x) = Vector{Float64}(x)
from_library_basis(nls, xl) = xl

end # module
