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
Gridap's reference FEs by a fixed reference-cell change of basis.  `LocalMaps()`
computes it once by evaluating Gridap's own dof functionals on the library's
basis functions, M[i,k] = σᵢ(ψₖ) (Gridap local dof i, library slot k):
  - u (Q2): the library slot (component c, node n) takes the Gridap dof with the
    same node and component, so M is a permutation and the values are unchanged;
  - j (RT1): the library's face functions carry no normal flux through any other
    face and its interior functions none through any face, so M is block
    triangular: 4 x 4 per face and 12 x 12 for the interior with a face coupling;
    a face's library values depend on that face's Gridap values only, the same
    from both cells sharing it;
  - p (dP1) and φ (dQ1): cell-own 4 x 4 and 8 x 8 maps.
Library slot k of a face or of the cell interior is given the global id of the
k-th Gridap dof owned by the same entity, so both vectors share Gridap's global
numbering and only the values are converted (`to_library_basis` /
`from_library_basis`, free and Dirichlet values alike).  The maps assume cells
whose RT face orientation agrees with the reference (Cartesian-type meshes, as
the Hunt and expansion meshers produce); other meshes would need Gridap's sign
flips applied per cell.

`GB300Objective` is a differentiable objective J(θ) = ∂J/∂x ⋅ x(θ) of the
Newton solution, θ = (Ha, cw, f_z per cell); its ChainRulesCore `rrule` calls
gbmhd_adjoint and maps dJ/dγ, dJ/dα, dJ/dβ to dJ/dHa for the scaling in use.

This file has not been executed in this build (no Julia toolchain); the C
entry points it binds are the ones the Python binding exercises.
"""
module GridapMHDGB300

using Gridap
using Gridap.FESpaces, Gridap.MultiField, Gridap.Algebra, Gridap.ReferenceFEs, Gridap.Geometry, Gridap.Fields
using LinearAlgebra
import ChainRulesCore
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

struct GbObjective
  dJdx::Ptr{Float64}
  n_theta_cells::Int32
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

mutable struct GB300NewtonSolver <: NonlinearSolver
  params::Dict{Symbol,Any}
  handle::Base.RefValue{Ptr{Cvoid}}
  keep::Vector{Any}
  trial::Any                   # the multi-field trial space (per-field cell dof ids)
  maps::LocalMaps              # Gridap ↔ library change of basis
  prm_template::GbParams       # the physical parameters passed at creation
  facet_cw::Vector{Float64}    # wall conductance per thin-wall facet (GB300Objective)
  fcell::Vector{Float64}       # [ncells][3] cellwise body force buffer (GB300Objective)
  ndofs::Int
end

function GB300NewtonSolver(op, params)
  h = Ref{Ptr{Cvoid}}(C_NULL)
  keep = Any[]
  mesh, dofs, prm, maps, facet_cw = extract(op, params, keep)
  GC.@preserve keep begin
    rc = ccall((:gbmhd_create, LIB), Cint, (Ref{Ptr{Cvoid}}, Ref{GbMesh}, Ref{GbDofMap}, Ref{GbParams}),
               h, mesh, dofs, prm)
  end
  rc == 0 || error("gbmhd_create failed ($rc): $(last_error(C_NULL))")
  s = GB300NewtonSolver(params, h, keep, get_trial(op), maps, prm, facet_cw, zeros(3 * mesh.ncells),
                        sum(dofs.nfree))
  finalizer(x -> ccall((:gbmhd_destroy, LIB), Cvoid, (Ptr{Cvoid},), x.handle[]), s)
  s
end

function f_cell_buffer!(nls::GB300NewtonSolver, fz)
  for c in eachindex(fz)
    nls.fcell[3c-2] = 0.0; nls.fcell[3c-1] = 0.0; nls.fcell[3c] = fz[c]
  end
  nls.fcell
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
  maps = LocalMaps()
  cell_dofs = Vector{Int32}(undef, 129 * ncells)
  nfree = zeros(Int64, 4); ndir = zeros(Int64, 4)
  dirv = Ptr{Float64}[C_NULL, C_NULL, C_NULL, C_NULL]
  for (f, Uf) in enumerate(U)
    ids = get_cell_dof_ids(Uf)
    nfree[f] = num_free_dofs(Uf)
    ndir[f] = num_dirichlet_dofs(Uf)
    # Dirichlet values in the library basis
    dv = to_library_values(maps, f, ids, Vector{Float64}(get_dirichlet_dof_values(Uf)), true)
    push!(keep, dv)
    dirv[f] = pointer(dv)
    off = SLOT_OFFSET[f]
    for c in 1:ncells, (k, p) in enumerate(maps.slot_to_dof[f])
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
  mesh, dofs, prm, maps, cw
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

# ---------------------------------------------------------------- change of basis (see module doc)
const SLOT_OFFSET = (0, 81, 85, 121)  # library slots of u, p, j, φ in a cell
L2(q, t) = q == 0 ? (2t - 1) * (t - 1) : q == 1 ? 4t * (1 - t) : t * (2t - 1)
L1(l, t) = l == 0 ? 1 - t : t

# The library's reference basis functions of each field, as Gridap fields, in slot order.
function library_fields(f)
  if f == 1      # u: component-major, n = a + 3b + 9c over the nodes {0, ½, 1}³
    [GenericField(x -> VectorValue(ntuple(i -> i == c + 1 ? L2(n % 3, x[1]) * L2((n ÷ 3) % 3, x[2]) * L2(n ÷ 9, x[3]) : 0.0, 3)))
     for c in 0:2 for n in 0:26]
  elseif f == 2  # p: 1 − ξ1 − ξ2 − ξ3, ξ1, ξ2, ξ3
    [GenericField(x -> 1 - x[1] - x[2] - x[3]), GenericField(x -> x[1]), GenericField(x -> x[2]),
     GenericField(x -> x[3])]
  elseif f == 3  # j: d*12 + q + 3*(l1 + 2*l2), ψ = L2_q(ξ_d) L1_l1(ξ_o1) L1_l2(ξ_o2) e_d
    fields = GenericField[]
    for b in 0:35
      d = b ÷ 12; r = b % 12; q = r % 3; l1 = (r ÷ 3) % 2; l2 = (r ÷ 3) ÷ 2
      o1 = d == 0 ? 1 : 0; o2 = d == 2 ? 1 : 2
      push!(fields, GenericField(x -> VectorValue(ntuple(i -> i == d + 1 ?
                    L2(q, x[d+1]) * L1(l1, x[o1+1]) * L1(l2, x[o2+1]) : 0.0, 3))))
    end
    fields
  else           # φ: Q1 nodal at the vertices a + 2b + 4c
    [GenericField(x -> L1(v & 1, x[1]) * L1((v >> 1) & 1, x[2]) * L1((v >> 2) & 1, x[3])) for v in 0:7]
  end
end

reference_fes() = (LagrangianRefFE(VectorValue{3,Float64}, HEX, 2), LagrangianRefFE(Float64, HEX, 1; space=:P),
                   RaviartThomasRefFE(Float64, HEX, 1), LagrangianRefFE(Float64, HEX, 1))

# σᵢ(ψₖ) with Gridap's dof functionals; the orientation of Gridap's result (dofs x fields or
# fields x dofs) is settled by the reproduction ψₖ(x) = Σᵢ M[i,k] φᵢ(x) at a test point.
function dof_matrix(reffe, fields)
  M = evaluate(get_dof_basis(reffe), fields)
  shp = get_shapefuns(reffe)
  x = [Point(0.31, 0.47, 0.73)]
  Φ = evaluate(shp, x)[1, :]          # φᵢ(x)
  Ψ = [evaluate(ψ, x)[1] for ψ in fields]
  ok(A) = all(k -> isapprox(Ψ[k], sum(A[i, k] * Φ[i] for i in eachindex(Φ)); atol=1e-12), eachindex(Ψ))
  ok(M) && return Matrix{Float64}(M)
  Mt = permutedims(M)
  ok(Mt) || error("GridapMHDGB300: cannot reproduce the library basis from Gridap's shape functions")
  Matrix{Float64}(Mt)
end

# The entity (vertex / edge / face / cell of HEX, Gridap numbering) that owns each local dof.
function dof_owner(reffe)
  own = get_face_own_dofs(reffe)
  owner = zeros(Int, num_dofs(reffe))
  for (e, ds) in enumerate(own), d in ds
    owner[d] = e
  end
  owner
end

# The HEX 2-face with the given axis (0-based) and side, as a Gridap entity number.
function hex_face_entity(axis, side)
  X = get_vertex_coordinates(HEX)
  fv = get_faces(HEX, 2, 0)
  off = num_faces(HEX, 0) + num_faces(HEX, 1)
  for (k, vs) in enumerate(fv)
    all(v -> X[v][axis+1] == side, vs) && return off + k
  end
  error("no face at axis $axis side $side")
end

struct LocalMaps
  slot_to_dof::NTuple{4,Vector{Int}}   # Gridap local dof of each library slot
  M::NTuple{4,Matrix{Float64}}          # σᵢ(ψₖ), rows Gridap local dofs, columns library slots
  blocks::NTuple{4,Vector{Vector{Int}}} # library slots per owning entity (a face, or the cell)
end

function LocalMaps()
  fes = reference_fes()
  slots = Vector{Vector{Int}}(undef, 4); Ms = Vector{Matrix{Float64}}(undef, 4)
  blks = Vector{Vector{Vector{Int}}}(undef, 4)
  for f in 1:4
    reffe = fes[f]
    M = dof_matrix(reffe, library_fields(f))
    owner = dof_owner(reffe)
    nd = num_dofs(reffe)
    s2d = zeros(Int, nd)
    if f == 1
      # node and component matching (M is a permutation)
      for k in 1:nd
        i = findfirst(i -> abs(M[i, k] - 1) < 1e-12, 1:nd)
        s2d[k] = i
      end
      blks[f] = [collect(1:nd)]
    elseif f == 3
      # face slots (q ∈ {0, 2}) ↔ the dofs owned by that face, interior slots ↔ the cell's
      groups = Dict{Int,Vector{Int}}()
      for b in 0:35
        d = b ÷ 12; q = (b % 12) % 3
        e = q == 1 ? num_faces(HEX) : hex_face_entity(d, q ÷ 2)
        push!(get!(groups, e, Int[]), b + 1)
      end
      for (e, ks) in groups
        ds = findall(==(e), owner)
        length(ds) == length(ks) || error("GridapMHDGB300: RT1 dof counts differ on entity $e")
        s2d[ks] .= ds
      end
      blks[f] = [ks for (e, ks) in sort(collect(groups); by=first)]  # faces first, the cell last
    else
      s2d .= 1:nd  # cell-own dofs: slot k ↔ Gridap dof k
      blks[f] = [collect(1:nd)]
    end
    slots[f] = s2d
    Ms[f] = M[s2d, :]  # rows in slot order: row k = the Gridap dof paired with slot k
  end
  LocalMaps(Tuple(slots), Tuple(Ms), Tuple(blks))
end

# Convert the values of one field between the bases, entity by entity (faces first, then the
# cell interior): Gridap values g = M c, so c_E = M_EE⁻¹ (g_E − Σ_{E' before E} M_EE' c_E').
# `ids` are Gridap's cell dof ids; with dirichlet, the values are the Dirichlet ones (ids < 0).
function convert_field(maps::LocalMaps, f, ids, v::Vector{Float64}, dirichlet::Bool, to_library::Bool)
  f == 1 && return copy(v)  # u: same values, the permutation is in the cell dof ids
  M = maps.M[f]; s2d = maps.slot_to_dof[f]; blks = maps.blocks[f]
  out = copy(v)
  done = falses(length(v))
  for cell_ids in ids
    gid = [cell_ids[s2d[k]] for k in 1:length(s2d)]     # global id of each library slot
    sel(k) = dirichlet ? gid[k] < 0 : gid[k] > 0
    pos(k) = dirichlet ? -gid[k] : gid[k]
    c = zeros(length(s2d))
    for (bi, ks) in enumerate(blks)
      all(sel, ks) || continue
      prev = reduce(vcat, blks[1:bi-1]; init=Int[])
      if to_library
        rhs = [v[pos(k)] for k in ks] .- M[ks, prev] * c[prev]
        c[ks] = M[ks, ks] \ rhs
        for (t, k) in enumerate(ks)
          p = pos(k)
          done[p] || (out[p] = c[ks][t]; done[p] = true)
        end
      else
        c[ks] = [v[pos(k)] for k in ks]
        g = M[ks, ks] * c[ks] .+ M[ks, prev] * c[prev]
        for (t, k) in enumerate(ks)
          p = pos(k)
          done[p] || (out[p] = g[t]; done[p] = true)
        end
      end
    end
  end
  out
end

to_library_values(maps, f, ids, v, dirichlet) = convert_field(maps, f, ids, v, dirichlet, true)

# Free vectors [u; p; j; φ] between Gridap's basis and the library's.
function convert_free(nls, x::AbstractVector, to_library::Bool)
  U = nls.trial
  out = Vector{Float64}(x)
  off = 0
  for (f, Uf) in enumerate(U)
    n = num_free_dofs(Uf)
    seg = out[off+1:off+n]
    out[off+1:off+n] = convert_field(nls.maps, f, get_cell_dof_ids(Uf), seg, false, to_library)
    off += n
  end
  out
end
to_library_basis(nls, x) = convert_free(nls, x, true)
from_library_basis(nls, xl) = convert_free(nls, xl, false)

# ---------------------------------------------------------------- differentiable objective
"""
    GB300Objective(nls, dJdx; Re, scaling=:cfd, base_params)

J(θ) = dJdx ⋅ x(θ), with x(θ) the Newton solution for θ = [Ha, cw, f_z per cell...] (the
f_z entries optional).  `scaling` is `:cfd` (γ = Ha²/Re, src/Applications/hunt.jl:125-128)
or `:mhd` (α = Re/Ha², β = 1/Ha², src/Applications/expansion.jl:113-123).  The rrule's
pullback calls gbmhd_adjoint at the solution and applies the chain rule for Ha.
"""
struct GB300Objective
  nls::Any
  dJdx::Vector{Float64}
  Re::Float64
  scaling::Symbol
end

function set_theta!(o::GB300Objective, θ)
  Ha, cw = θ[1], θ[2]
  p = o.nls.prm_template
  α, β, γ = o.scaling == :cfd ? (1.0, 1 / o.Re, Ha^2 / o.Re) : (o.Re / Ha^2, 1 / Ha^2, 1.0)
  fill!(o.nls.facet_cw, cw)
  fz = length(θ) > 2 ? θ[3:end] : nothing
  fcell = fz === nothing ? C_NULL : pointer(f_cell_buffer!(o.nls, fz))
  prm = GbParams(α, β, γ, p.sigma, p.B, p.f, p.g, p.zeta_u, p.zeta_j, p.convection, fcell, p.nfacets,
                 p.facet_cell, p.facet_lface, p.facet_tau, pointer(o.nls.facet_cw), p.facet_jw, p.facet_phi0)
  GC.@preserve o begin
    check(ccall((:gbmhd_set_params, LIB), Cint, (Ptr{Cvoid}, Ref{GbParams}), o.nls.handle[], prm),
          o.nls.handle[], "gbmhd_set_params")
  end
end

function solve_library(o::GB300Objective, θ)
  set_theta!(o, θ)
  x = zeros(o.nls.ndofs)
  s = o.nls.params[:solver]
  opts = GbSolveOpts(s[:precision] == :mixed ? 1 : 0, s[:niter], s[:rtol], s[:atol], s[:niter_ls],
                     s[:max_linear], s[:linear_rtol], 0, s[:preconditioner] == :monolithic ? 0 : 1)
  rep = GbReport()
  check(ccall((:gbmhd_newton_solve, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ref{GbSolveOpts}, Ref{GbReport}),
              o.nls.handle[], x, opts, rep), o.nls.handle[], "gbmhd_newton_solve")
  x, opts
end

(o::GB300Objective)(θ) = dot(o.dJdx, first(solve_library(o, θ)))

function ChainRulesCore.rrule(o::GB300Objective, θ::AbstractVector)
  x, opts = solve_library(o, θ)
  J = dot(o.dJdx, x)
  function pullback(J̄)
    ncell = length(θ) - 2
    dJ = zeros(4 + max(ncell, 0))
    obj = GbObjective(pointer(o.dJdx), Int32(ncell > 0 ? 1 : 0))
    rep = GbReport()
    GC.@preserve o x dJ begin
      check(ccall((:gbmhd_adjoint, LIB), Cint,
                  (Ptr{Cvoid}, Ptr{Float64}, Ref{GbObjective}, Ref{GbSolveOpts}, Ptr{Float64}, Int64, Ptr{Float64},
                   Ref{GbReport}), o.nls.handle[], x, obj, opts, dJ, length(dJ), C_NULL, rep),
            o.nls.handle[], "gbmhd_adjoint")
    end
    Ha = θ[1]
    # dJ = [dJ/dγ, dJ/dcw, dJ/dα, dJ/dβ, dJ/df_z...]
    dHa = o.scaling == :cfd ? dJ[1] * 2Ha / o.Re : -2 / Ha^3 * (o.Re * dJ[3] + dJ[4])
    grad = vcat(dHa, dJ[2], ncell > 0 ? dJ[5:end] : Float64[])
    (ChainRulesCore.NoTangent(), J̄ .* grad)
  end
  J, pullback
end

end # module
