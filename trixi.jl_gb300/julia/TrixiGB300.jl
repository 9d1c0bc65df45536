# TrixiGB300.jl -- Julia side of the drop-in: a device backend for Trixi.jl's
# TreeMesh DGSEM Euler path that forwards to libtrixi_gb300.so through ccall.
#
# The seam is rhs_hyperbolic!(backend, du, u, t, mesh, equations, ...)
# (src/solvers/dgsem_tree/dg_2d.jl:113), selected by trixi_backend(u)
# (src/auxiliary/containers.jl:278); the KernelAbstractions backend plugs in
# at the same place (src/solvers/dgsem_p4est/dg_2d_gpu.jl:8).  The ODE state
# is a GB300Array (device memory owned by the library), so that
# `rhs_hyperbolic!(du_ode, u_ode, semi, t)`
# (semidiscretization_hyperbolic.jl:578-597) finds the backend through
# trixi_backend(u), and OrdinaryDiffEq's CarpenterKennedy2N54 drives it
# unchanged: its broadcasts (tmp = A tmp + dt du; u = u + B tmp) lower to
# the library's tg_lincomb.
#
# Julia is not installed where this repository is tested.  The calling
# convention -- the tg_config built from Trixi's own arrays, library-owned
# device vectors, tg_rhs on them, the 2N broadcasts through tg_lincomb -- is
# exercised from C by tests/c/shim_driver.c (tests/test_gpu_shim_abi.py).
module TrixiGB300

using Trixi
using Trixi: True, False
using SciMLBase: ODEProblem

const lib = joinpath(@__DIR__, "..", "_build", "libtrixi_gb300.so")

# tg_config, include/trixi_gb300.h (field order and types must match)
struct TgConfig
    ndims::Int32
    polydeg::Int32
    nelements::Int64
    ninterfaces::Int64
    gamma::Float64
    volume_integral::Int32
    volume_flux::Int32
    surface_flux::Int32
    volume_flux_fv::Int32
    alpha_max::Float64
    alpha_min::Float64
    alpha_smooth::Int32
    source_terms::Int32
    precision::Int32
    device::Int32
    nodes::Ptr{Float64}
    weights::Ptr{Float64}
    inverse_weights::Ptr{Float64}
    derivative_hat::Ptr{Float64}
    derivative_split::Ptr{Float64}
    inverse_vandermonde_legendre::Ptr{Float64}
    neighbor_ids::Ptr{Int64}
    orientations::Ptr{Int64}
    inverse_jacobian::Ptr{Float64}
    node_coordinates::Ptr{Float64}
    elements_per_block::Int32
    boundary_conditions::NTuple{6, Int32}  # per direction: 0 periodic, 1 Dirichlet, 2 slip wall
    boundary_value_function::Int32         # tg_initial_condition of Dirichlet faces
    boundary_value_params::NTuple{4, Float64}
    nmortars::Int64                        # cache.mortars (L2 mortars)
    mortar_neighbor_ids::Ptr{Int64}
    mortar_large_sides::Ptr{Int64}
    mortar_orientations::Ptr{Int64}
    mortar_forward_upper::Ptr{Float64}     # dg.mortar
    mortar_forward_lower::Ptr{Float64}
    mortar_reverse_upper::Ptr{Float64}
    mortar_reverse_lower::Ptr{Float64}
    mesh_type::Int32                        # 0 TreeMesh, 1 curvilinear 2D brick
    contravariant_vectors::Ptr{Float64}     # [2, 2, n, n, E] (curvilinear)
end

const TG_VOLUME_WEAK_FORM, TG_VOLUME_FLUX_DIFFERENCING, TG_VOLUME_SHOCK_CAPTURING_HG = 0, 1, 2
const TG_FLUX_CENTRAL, TG_FLUX_RANOCHA, TG_FLUX_SHIMA_ETAL = 0, 1, 2
const TG_FLUX_LAX_FRIEDRICHS, TG_FLUX_LAX_FRIEDRICHS_NAIVE, TG_FLUX_HLLC = 3, 4, 5
const TG_FLUX_CHANDRASHEKAR, TG_FLUX_HLLE = 6, 7

flux_code(::typeof(Trixi.flux_central)) = TG_FLUX_CENTRAL
flux_code(::typeof(Trixi.flux_ranocha)) = TG_FLUX_RANOCHA
flux_code(::typeof(Trixi.flux_shima_etal)) = TG_FLUX_SHIMA_ETAL
flux_code(::typeof(Trixi.flux_hllc)) = TG_FLUX_HLLC
flux_code(::typeof(Trixi.flux_chandrashekar)) = TG_FLUX_CHANDRASHEKAR
flux_code(f::Trixi.FluxHLL) = f.min_max_speed === Trixi.min_max_speed_einfeldt ? TG_FLUX_HLLE :
                              error("FluxHLL: only min_max_speed_einfeldt (flux_hlle) is on the GPU path")
function flux_code(f::Trixi.FluxLaxFriedrichs)
    f.dissipation.max_abs_speed === Trixi.max_abs_speed_naive ?
    TG_FLUX_LAX_FRIEDRICHS_NAIVE : TG_FLUX_LAX_FRIEDRICHS
end

source_code(::Nothing) = 0
source_code(::typeof(Trixi.source_terms_convergence_test)) = 1

struct GB300Backend end

mutable struct GB300Context
    ptr::Ptr{Cvoid}
end

function last_error(ctx::Ptr{Cvoid})
    buf = Vector{UInt8}(undef, 1024)
    ccall((:tg_last_error, lib), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), ctx, buf, length(buf))
    return unsafe_string(pointer(buf))
end

check(rc, ctx = C_NULL) = rc == 0 || error("libtrixi_gb300: " * last_error(ctx))

function volume_codes(vi::VolumeIntegralWeakForm, surface_flux)
    return (TG_VOLUME_WEAK_FORM, TG_FLUX_CENTRAL, flux_code(surface_flux), 0.5, 0.001, true)
end
function volume_codes(vi::VolumeIntegralFluxDifferencing, surface_flux)
    return (TG_VOLUME_FLUX_DIFFERENCING, flux_code(vi.volume_flux), flux_code(surface_flux),
            0.5, 0.001, true)
end
function volume_codes(vi::Trixi.VolumeIntegralShockCapturingHGType, surface_flux)
    ind = vi.indicator
    return (TG_VOLUME_SHOCK_CAPTURING_HG, flux_code(vi.volume_integral_blend_high_order.volume_flux),
            flux_code(vi.volume_integral_blend_low_order.volume_flux_fv),
            ind.alpha_max, ind.alpha_min, ind.alpha_smooth)
end

"""
    create_context(semi; precision = 0, device = 0)

Builds a device context from a `SemidiscretizationHyperbolic` on a periodic
`TreeMesh` with `DGSEM` (precision 0 = FP64, 1 = mixed FP32/float-float).
"""
# tg_config of a semidiscretization; the pointers stay valid while `semi` is
# preserved (GC.@preserve) by the caller.
function config(semi, precision, device)
    (; mesh, equations, solver, cache, source_terms) = semi
    mesh isa Union{Trixi.StructuredMesh{2}, Trixi.P4estMesh{2}, Trixi.StructuredMesh{3}} &&
        return curved_config(semi, precision, device)
    b = solver.basis
    vi, vf, sf_fv, amax, amin, asmooth = volume_codes(solver.volume_integral,
                                                      solver.surface_integral.surface_flux)
    sf = flux_code(solver.surface_integral.surface_flux)
    return TgConfig(ndims(mesh), Trixi.polydeg(solver), nelements(solver, cache),
                    ninterfaces(solver, cache), equations.gamma, vi, vf, sf,
                    vi == TG_VOLUME_SHOCK_CAPTURING_HG ? sf_fv : sf, amax, amin, asmooth,
                    source_code(source_terms), precision, device,
                    pointer(b.nodes), pointer(b.weights), pointer(b.inverse_weights),
                    pointer(b.derivative_hat), pointer(b.derivative_split),
                    pointer(b.inverse_vandermonde_legendre),
                    pointer(cache.interfaces.neighbor_ids),
                    pointer(cache.interfaces.orientations),
                    pointer(cache.elements.inverse_jacobian),
                    pointer(cache.elements.node_coordinates), 0,
                    boundary_codes(semi.boundary_conditions, ndims(mesh)),
                    boundary_value_code(semi.boundary_conditions)...,
                    mortar_fields(solver, cache)...,
                    Int32(0), Ptr{Float64}(C_NULL))
end

# Interfaces of a curvilinear brick as (element on the negative side, element on
# the positive side) pairs and directions, 1-based like Trixi's arrays.  The
# arrays are kept in `CURVED_KEEP` while the config is in use.
const CURVED_KEEP = IdDict{Any, Any}()
function curved_interfaces(mesh::Trixi.StructuredMesh{2}, cache)
    ln = cache.elements.left_neighbors            # [2, E]: element across the face at -dir (0: boundary)
    E = size(ln, 2)
    keep = [(d, e) for e in 1:E for d in 1:2 if ln[d, e] > 0]
    return [ln[d, e] for (d, e) in keep], [e for (d, e) in keep], [d for (d, e) in keep]
end
function curved_interfaces(mesh::Trixi.StructuredMesh{3}, cache)
    ln = cache.elements.left_neighbors            # [3, E]: element across the face at -dir
    E = size(ln, 2)
    keep = [(d, e) for e in 1:E for d in 1:3 if ln[d, e] > 0]
    return [ln[d, e] for (d, e) in keep], [e for (d, e) in keep], [d for (d, e) in keep]
end
function curved_interfaces(mesh::Trixi.P4estMesh{2}, cache)
    # primary side at :end of its face coordinate = negative side of the interface
    ids, ni = cache.interfaces.neighbor_ids, cache.interfaces.node_indices
    neg, pos, dir = Int[], Int[], Int[]
    for i in axes(ids, 2)
        d = Trixi.indices2direction(ni[1, i])      # 1..4: -x, +x, -y, +y of the primary
        push!(neg, iseven(d) ? ids[1, i] : ids[2, i])
        push!(pos, iseven(d) ? ids[2, i] : ids[1, i])
        push!(dir, (d + 1) >> 1)
    end
    return neg, pos, dir
end

function curved_config(semi, precision, device)
    (; mesh, equations, solver, cache, source_terms) = semi
    b = solver.basis
    neg, pos, dir = curved_interfaces(mesh, cache)
    nb = permutedims(hcat(neg, pos))           # [2, I], column-major as Trixi's
    ori = Vector{Int}(dir)
    CURVED_KEEP[semi] = (nb, ori)
    vi, vf, sf_fv, amax, amin, asmooth = volume_codes(solver.volume_integral,
                                                      solver.surface_integral.surface_flux)
    sf = flux_code(solver.surface_integral.surface_flux)
    return TgConfig(ndims(mesh), Trixi.polydeg(solver), nelements(solver, cache), length(ori),
                    equations.gamma, vi, vf, sf, sf, amax, amin, asmooth,
                    source_code(source_terms), precision, device,
                    pointer(b.nodes), pointer(b.weights), pointer(b.inverse_weights),
                    pointer(b.derivative_hat), pointer(b.derivative_split),
                    pointer(b.inverse_vandermonde_legendre), pointer(nb), pointer(ori),
                    pointer(cache.elements.inverse_jacobian),      # [n, n(, n), E]
                    pointer(cache.elements.node_coordinates), 0,
                    boundary_codes(semi.boundary_conditions, ndims(mesh)),
                    boundary_value_code(semi.boundary_conditions)...,
                    Int64(0), Ptr{Int64}(C_NULL), Ptr{Int64}(C_NULL), Ptr{Int64}(C_NULL),
                    Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL),
                    Ptr{Float64}(C_NULL),
                    Int32(1), pointer(cache.elements.contravariant_vectors))
end

# cache.mortars / dg.mortar of a TreeMesh with L2 mortars (none: zero and NULL)
function mortar_fields(solver, cache)
    m = solver.mortar
    nm = hasproperty(cache, :mortars) ? Trixi.nmortars(cache.mortars) : 0
    nm == 0 && return (Int64(0), Ptr{Int64}(C_NULL), Ptr{Int64}(C_NULL), Ptr{Int64}(C_NULL),
                       Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL),
                       Ptr{Float64}(C_NULL))
    return (Int64(nm), pointer(cache.mortars.neighbor_ids), pointer(cache.mortars.large_sides),
            pointer(cache.mortars.orientations), pointer(m.forward_upper),
            pointer(m.forward_lower), pointer(m.reverse_upper), pointer(m.reverse_lower))
end

# boundary_conditions of the semidiscretization (digested: one per direction
# for non-periodic meshes) as tg_boundary codes
bc_code(::Trixi.BoundaryConditionPeriodic) = Int32(0)
bc_code(::Trixi.BoundaryConditionDirichlet) = Int32(1)
bc_code(::typeof(Trixi.boundary_condition_slip_wall)) = Int32(2)
boundary_codes(bcs::Trixi.BoundaryConditionPeriodic, nd) = ntuple(_ -> Int32(0), 6)
boundary_codes(bcs::NamedTuple, nd) = ntuple(k -> k <= 2nd ? bc_code(bcs[k]) : Int32(0), 6)
# Non-periodic P4estMesh bricks carry their boundaries by name
# (UnstructuredSortedBoundaryTypes); the library takes one condition per
# direction of a TreeMesh or StructuredMesh only.
boundary_codes(bcs, nd) =
    error("TrixiGB300: boundary conditions of type $(typeof(bcs)) (for instance a " *
          "non-periodic P4estMesh) are not on the GPU path; use a periodic P4estMesh or a " *
          "StructuredMesh with one condition per direction")

# Dirichlet values: the initial conditions the device evaluates
ic_code(::typeof(Trixi.initial_condition_constant)) = Int32(0)
ic_code(::typeof(Trixi.initial_condition_convergence_test)) = Int32(1)
ic_code(::typeof(Trixi.initial_condition_weak_blast_wave)) = Int32(3)
function boundary_value_code(bcs)
    for bc in (bcs isa NamedTuple ? values(bcs) : (bcs,))
        bc isa Trixi.BoundaryConditionDirichlet &&
            return ic_code(bc.boundary_value_function), (0.0, 0.0, 0.0, 0.0)
    end
    return Int32(0), (0.0, 0.0, 0.0, 0.0)
end

function create_context(semi; precision = 0, device = 0)
    GC.@preserve semi begin
        cfg = config(semi, precision, device)
        out = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:tg_ctx_create, lib), Cint, (Ref{TgConfig}, Ref{Ptr{Cvoid}}), cfg, out))
    end
    ctx = GB300Context(out[])
    finalizer(c -> ccall((:tg_ctx_destroy, lib), Cint, (Ptr{Cvoid},), c.ptr), ctx)
    return ctx
end

"""
    rhs!(ctx, du, u, t)

`rhs_hyperbolic!` for device vectors `du`, `u` (Trixi layout, Float64).
"""
function rhs!(ctx::GB300Context, du, u, t)
    check(ccall((:tg_rhs, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Cdouble),
                ctx.ptr, pointer(du), pointer(u), t), ctx.ptr)
    return nothing
end

# ---- the ODE state in device memory ------------------------------------------------
"""
    GB300Array <: AbstractVector{Float64}

A flat `u_ode` vector in Trixi's layout that lives in device memory owned by
the library (tg_vector_create), tied to the context it is used with.  Scalar
indexing is not supported; `copyto!` moves data to and from host `Vector`s,
and broadcasts that are linear combinations of at most two GB300Arrays with
scalar coefficients (what low-storage Runge-Kutta methods use) run on the
device through tg_lincomb.
"""
mutable struct GB300Array <: AbstractVector{Float64}
    ptr::Ptr{Float64}
    len::Int
    ctx::GB300Context
    function GB300Array(ctx::GB300Context, len::Integer)
        p = Ref{Ptr{Float64}}(C_NULL)
        check(ccall((:tg_vector_create, lib), Cint, (Ptr{Cvoid}, Int64, Ref{Ptr{Float64}}),
                    ctx.ptr, len, p), ctx.ptr)
        a = new(p[], Int(len), ctx)
        finalizer(a) do x
            ctx.ptr == C_NULL ||
                ccall((:tg_vector_destroy, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx.ptr, x.ptr)
        end
        return a
    end
end

Base.size(a::GB300Array) = (a.len,)
Base.pointer(a::GB300Array) = a.ptr
Base.IndexStyle(::Type{GB300Array}) = IndexLinear()
Base.getindex(::GB300Array, ::Int) =
    error("GB300Array: scalar indexing of device memory; copy it to a Vector first")
Base.setindex!(::GB300Array, v, ::Int) =
    error("GB300Array: scalar indexing of device memory; copy a Vector into it instead")
Base.similar(a::GB300Array) = GB300Array(a.ctx, a.len)
Base.similar(a::GB300Array, ::Type{Float64}) = similar(a)
Base.similar(a::GB300Array, ::Type{Float64}, dims::Tuple{Int}) = GB300Array(a.ctx, dims[1])

function vector_copy!(dst::Ptr, src::Ptr, n, kind, ctx)
    check(ccall((:tg_vector_copy, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int32),
                ctx.ptr, dst, src, n, kind), ctx.ptr)
end
function Base.copyto!(dst::GB300Array, src::Vector{Float64})
    GC.@preserve src vector_copy!(dst.ptr, pointer(src), dst.len, 0, dst.ctx)
    return dst
end
function Base.copyto!(dst::Vector{Float64}, src::GB300Array)
    GC.@preserve dst vector_copy!(pointer(dst), src.ptr, src.len, 1, src.ctx)
    return dst
end
function Base.copyto!(dst::GB300Array, src::GB300Array)
    vector_copy!(dst.ptr, src.ptr, dst.len, 2, dst.ctx)
    return dst
end
Base.Array(a::GB300Array) = copyto!(Vector{Float64}(undef, a.len), a)

# broadcasts: sum of scalar multiples of at most two GB300Arrays
Base.BroadcastStyle(::Type{GB300Array}) = Broadcast.ArrayStyle{GB300Array}()
function Base.similar(bc::Broadcast.Broadcasted{Broadcast.ArrayStyle{GB300Array}},
                      ::Type{Float64})
    return similar(find_gb300(bc))
end
find_gb300(bc::Broadcast.Broadcasted) = find_gb300(bc.args)
find_gb300(args::Tuple) = (a = find_gb300(first(args)); a === nothing ? find_gb300(Base.tail(args)) : a)
find_gb300(::Tuple{}) = nothing
find_gb300(a::GB300Array) = a
find_gb300(x) = nothing

# terms!(terms, expr, c): add c * expr to the list of (coefficient, array) terms
terms!(t, a::GB300Array, c) = (push!(t, (c, a)); t)
terms!(t, x::Number, c) = error("GB300Array broadcast: a scalar term is not a linear combination")
function terms!(t, bc::Broadcast.Broadcasted, c)
    f, args = bc.f, bc.args
    if f === (+) && length(args) == 2
        terms!(t, args[1], c); terms!(t, args[2], c)
    elseif f === (-) && length(args) == 2
        terms!(t, args[1], c); terms!(t, args[2], -c)
    elseif f === (-) && length(args) == 1
        terms!(t, args[1], -c)
    elseif f === (*) && length(args) == 2 && args[1] isa Number
        terms!(t, args[2], c * args[1])
    elseif f === (*) && length(args) == 2 && args[2] isa Number
        terms!(t, args[1], c * args[2])
    elseif f === identity && length(args) == 1
        terms!(t, args[1], c)
    else
        error("GB300Array broadcast: only linear combinations of device vectors run on the GPU")
    end
    return t
end
terms!(t, r::Base.RefValue, c) = terms!(t, r[], c)

function Base.copyto!(dst::GB300Array,
                      bc::Broadcast.Broadcasted{Broadcast.ArrayStyle{GB300Array}})
    t = terms!(Tuple{Float64, GB300Array}[], bc, 1.0)
    merged = Dict{Ptr{Float64}, Tuple{Float64, GB300Array}}()
    for (c, a) in t
        prev = get(merged, a.ptr, (0.0, a))
        merged[a.ptr] = (prev[1] + c, a)
    end
    length(merged) <= 2 ||
        error("GB300Array broadcast: at most two device vectors per linear combination")
    (c1, x), rest = first(values(merged)), collect(values(merged))[2:end]
    c2, y = isempty(rest) ? (0.0, nothing) : rest[1]
    check(ccall((:tg_lincomb, lib), Cint,
                (Ptr{Cvoid}, Int64, Ptr{Float64}, Cdouble, Ptr{Float64}, Cdouble, Ptr{Float64}),
                dst.ctx.ptr, dst.len, dst.ptr, c1, x.ptr, c2,
                y === nothing ? Ptr{Float64}(C_NULL) : y.ptr), dst.ctx.ptr)
    return dst
end

# ---- the backend: Trixi dispatches rhs_hyperbolic! and max_dt on it ---------------
Trixi.trixi_backend(::GB300Array) = GB300Backend()
# the flat device vector is passed on as it is: the library reads Trixi's layout
Trixi.wrap_array(u_ode::GB300Array, mesh, equations, dg::DGSEM, cache) = u_ode

function Trixi.rhs_hyperbolic!(::GB300Backend, du::GB300Array, u::GB300Array, t,
                               mesh::Union{TreeMesh, StructuredMesh, P4estMesh}, equations,
                               boundary_conditions, source_terms, dg::DGSEM, cache)
    rhs!(u.ctx, du, u, t)
    return nothing
end

# StepsizeCallback: max_dt without the CFL factor, on the device
function Trixi.max_dt(u::GB300Array, t, mesh::Union{TreeMesh, StructuredMesh, P4estMesh},
                      constant_speed::False, equations, dg::DG, cache)
    dt = Ref{Cdouble}(0)
    check(ccall((:tg_max_dt, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ref{Cdouble}),
                u.ctx.ptr, u.ptr, dt), u.ctx.ptr)
    return dt[]
end

"""
    semidiscretize_gb300(semi, tspan; precision = 0, device = 0)

`semidiscretize(semi, tspan)` with the state on the GB300: creates the
device context of `semi` (kept alive with the returned problem's initial
state), evaluates the initial condition on the host as Trixi does and uploads
it into a GB300Array.  The ODEProblem's right-hand side is Trixi's own
`rhs!`, which reaches the library through trixi_backend(u).
"""
function semidiscretize_gb300(semi::SemidiscretizationHyperbolic, tspan;
                              precision = 0, device = 0)
    ctx = create_context(semi; precision, device)
    u0_host = Trixi.compute_coefficients(first(tspan), semi)
    u0 = copyto!(GB300Array(ctx, length(u0_host)), u0_host)
    return ODEProblem(Trixi.rhs!, u0, tspan, semi)
end

upload!(ctx::GB300Context, u::Vector{Float64}) =
    check(ccall((:tg_upload_state, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx.ptr, u), ctx.ptr)
download!(u::Vector{Float64}, ctx::GB300Context) =
    check(ccall((:tg_download_state, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx.ptr, u), ctx.ptr)

"""
    step_to!(ctx, t0, t_end, cfl; max_steps)

CarpenterKennedy2N54 with StepsizeCallback(cfl) semantics on the device (CUDA
graphs); returns the reached time and the number of steps.
"""
function step_to!(ctx::GB300Context, t0, t_end, cfl; max_steps = typemax(Int64))
    t = Ref{Cdouble}(t0)
    n = Ref{Int64}(0)
    check(ccall((:tg_step, lib), Cint,
                (Ptr{Cvoid}, Int64, Cdouble, Cdouble, Ref{Cdouble}, Ref{Int64}),
                ctx.ptr, max_steps, cfl, t_end, t, n), ctx.ptr)
    return t[], n[]
end

function max_dt(ctx::GB300Context)
    dt = Ref{Cdouble}(0)
    check(ccall((:tg_max_dt, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ref{Cdouble}),
                ctx.ptr, C_NULL, dt), ctx.ptr)
    return dt[]
end

"""
    entropy_timederivative(ctx, t)

`analyze(entropy_timederivative, du, u, t, ...)` of the device state
(analysis_dg2d.jl:460-472): the normalised integral of cons2entropy(u) . rhs(u).
"""
function entropy_timederivative(ctx::GB300Context, t)
    out = Ref{Cdouble}(0)
    check(ccall((:tg_entropy_timederivative, lib), Cint, (Ptr{Cvoid}, Cdouble, Ref{Cdouble}),
                ctx.ptr, t, out), ctx.ptr)
    return out[]
end

"""
    autotune!(ctx; iters = 20)

Times every elements-per-block choice of the element kernel on the uploaded
state (which it leaves unchanged) and keeps the fastest; returns it and the
time per stage in ms.
"""
function autotune!(ctx::GB300Context; iters = 20)
    epb = Ref{Int32}(0)
    ms = Ref{Cdouble}(0)
    check(ccall((:tg_ctx_autotune, lib), Cint, (Ptr{Cvoid}, Int32, Ref{Int32}, Ref{Cdouble}),
                ctx.ptr, iters, epb, ms), ctx.ptr)
    return epb[], ms[]
end

# ---- batched ensembles: many 2D semidiscretizations stepped together -------------
mutable struct GB300Ensemble
    ptr::Ptr{Cvoid}
end

function ensemble_error(ens::Ptr{Cvoid})
    buf = Vector{UInt8}(undef, 1024)
    ccall((:tg_ensemble_last_error, lib), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), ens, buf,
          length(buf))
    return unsafe_string(pointer(buf))
end

"""
    create_ensemble(semis; threads_per_block = 0, device = 0)

One persistent launch per 2N stage and one CUDA graph per step for all of
`semis` (2D, polydeg 2..4, mixed precision, one solver type).
"""
function create_ensemble(semis; threads_per_block = 0, device = 0)
    GC.@preserve semis begin
        cfgs = [config(semi, 1, device) for semi in semis]
        out = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:tg_ensemble_create, lib), Cint, (Ptr{TgConfig}, Int32, Int32, Ref{Ptr{Cvoid}}),
                   cfgs, length(cfgs), threads_per_block, out)
        rc == 0 || error(ensemble_error(C_NULL))
    end
    ens = GB300Ensemble(out[])
    finalizer(e -> ccall((:tg_ensemble_destroy, lib), Cint, (Ptr{Cvoid},), e.ptr), ens)
    return ens
end

"""
    instance(ens, i)

Context of instance i (1-based), owned by the ensemble: `upload!`,
`download!` and the analysis calls work on it.
"""
function instance(ens::GB300Ensemble, i)
    p = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:tg_ensemble_context, lib), Cint, (Ptr{Cvoid}, Int32, Ref{Ptr{Cvoid}}), ens.ptr,
               i - 1, p)
    rc == 0 || error(ensemble_error(ens.ptr))
    return GB300Context(p[])  # no finalizer: the ensemble owns it
end

"""
    step_to!(ens, t, t_end, cfl; max_steps)

Every instance from its own `t[i]` with its own StepsizeCallback(cfl) step
size; updates `t` and returns the step counts.
"""
function step_to!(ens::GB300Ensemble, t::Vector{Float64}, t_end, cfl; max_steps = typemax(Int64))
    steps = zeros(Int64, length(t))
    rc = ccall((:tg_ensemble_step, lib), Cint,
               (Ptr{Cvoid}, Int64, Cdouble, Cdouble, Ptr{Cdouble}, Ptr{Int64}),
               ens.ptr, max_steps, cfl, t_end, t, steps)
    rc == 0 || error(ensemble_error(ens.ptr))
    return steps
end

"""
    amr_indicator(ctx, indicator)

The values ControllerThreeLevel compares with its thresholds, computed on the
device in FP64: `IndicatorHennemannGassner` (its alpha_max, alpha_min,
alpha_smooth; variable density_pressure or density) or `IndicatorMax`.
"""
function amr_indicator(ctx::GB300Context, ind::IndicatorHennemannGassner, nelements)
    out = zeros(Float64, nelements)
    variable = ind.variable === Trixi.density ? Int32(1) : Int32(0)
    check(ccall((:tg_amr_indicator, lib), Cint,
                (Ptr{Cvoid}, Cdouble, Cdouble, Int32, Int32, Ptr{Float64}),
                ctx.ptr, ind.alpha_max, ind.alpha_min, Int32(ind.alpha_smooth), variable, out),
          ctx.ptr)
    return out
end
function amr_indicator(ctx::GB300Context, ind::Trixi.IndicatorMax, nelements)
    out = zeros(Float64, nelements)
    variable = ind.variable === Trixi.density_pressure ? Int32(0) : Int32(1)
    check(ccall((:tg_amr_indicator_max, lib), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}),
                ctx.ptr, variable, out), ctx.ptr)
    return out
end

"""
    adapt_state!(new_ctx, old_ctx, source_element, kind, adaptor)

The solution transfer of refine!/coarsen! (amr_dg2d.jl) on the device, from
the context of the mesh before adaptation into the context of the adapted
mesh.  `source_element` (0-based) and `kind` (0 copy, 1 + child, -1 coarsen)
describe each new element; `adaptor` is the solver's LobattoLegendreAdaptorL2.
"""
function adapt_state!(new::GB300Context, old::GB300Context, source_element::Vector{Int64},
                      kind::Vector{Int8}, a)
    check(ccall((:tg_adapt_state, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Ptr{Int8}, Ptr{Float64}, Ptr{Float64},
                 Ptr{Float64}, Ptr{Float64}),
                new.ptr, old.ptr, source_element, kind, a.forward_upper, a.forward_lower,
                a.reverse_upper, a.reverse_lower), new.ptr)
    return new
end

end # module
