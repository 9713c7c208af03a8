# TrixiGB300.jl -- ccall glue that routes TrixiCUDA.jl's rhs path to
# libtrixi_b200.so (the GB300 / sm_103a C ABI declared in include/trixi_b200.h).
#
# This file is the Julia side of the drop-in boundary: it keeps the
# reference's public API (`DGSEMGPU`, `SemidiscretizationHyperbolicGPU`,
# `semidiscretizeGPU`, `rhs_gpu!`, src/TrixiCUDA.jl:70-73) and replaces the
# bodies of `rhs_gpu!` (src/solvers/solvers.jl:18-31) and of the `cuda_*`
# stage launchers (src/solvers/dg_{1,2,3}d.jl) by calls into the library.
# Julia is not installed where this library is built and tested, so this file
# has not been executed; the same entry points are exercised from Python
# (trixicuda/_lib.py) by the test suite.
module TrixiGB300

using CUDA
using Trixi
using ChainRulesCore

const libtrixi = get(ENV, "TRIXI_B200_LIB", joinpath(@__DIR__, "..", "_build", "libtrixi_b200.so"))

# enum values of include/trixi_b200.h
const EQ_LINEAR_ADVECTION = Int32(0)
const EQ_COMPRESSIBLE_EULER = Int32(1)
const EQ_IDEAL_GLM_MHD = Int32(2)
const VOLUME_WEAK_FORM = Int32(0)
const VOLUME_FLUX_DIFFERENCING = Int32(1)
const VOLUME_SHOCK_CAPTURING_HG = Int32(2)
const FLUX_LAX_FRIEDRICHS = Int32(0)
const FLUX_RANOCHA = Int32(1)
const FLUX_CENTRAL = Int32(2)
const FLUX_HINDENLANG_GASSNER = Int32(4)
const FLUX_SHIMA_ETAL = Int32(5)
const FLUX_HLL = Int32(6)
const FLUX_HLLE = Int32(7)
const SOURCE_NONE = Int32(0)
const SOURCE_CONVERGENCE_TEST = Int32(1)
const SOURCE_EOC_TEST_EULER = Int32(2)

# Source terms cross the C ABI as enums: the library has device code for
# these two Trixi functions only; any other Julia callable is refused.
function source_code(source_terms)
    source_terms === nothing && return SOURCE_NONE
    source_terms === Trixi.source_terms_convergence_test && return SOURCE_CONVERGENCE_TEST
    source_terms === Trixi.source_terms_eoc_test_euler && return SOURCE_EOC_TEST_EULER
    error("libtrixi_b200: source terms $(source_terms) have no device code in the library " *
          "(supported: source_terms_convergence_test, source_terms_eoc_test_euler)")
end
const NONCONSERVATIVE_NONE = Int32(0)
const NONCONSERVATIVE_POWELL = Int32(1)

# mirror of trixi_problem_desc (field order and types must match the C struct)
mutable struct ProblemDesc
    struct_size::Int32
    ndims::Int32
    polydeg::Int32
    nvars::Int32
    equation::Int32
    volume_integral::Int32
    volume_flux::Int32
    surface_flux::Int32
    volume_flux_fv::Int32
    precision::Int32
    gamma::Float64
    advection_velocity::NTuple{3, Float64}
    alpha_max::Float64
    alpha_min::Float64
    alpha_smooth::Int32
    indicator_variable::Int32
    nelements::Int64
    inverse_jacobian::Ptr{Float64}
    ninterfaces::Int64
    interface_neighbor_ids::Ptr{Int64}
    interface_orientations::Ptr{Int64}
    nboundaries::Int64
    nmortars::Int64
    mortar_neighbor_ids::Ptr{Int64}
    mortar_large_sides::Ptr{Int64}
    mortar_orientations::Ptr{Int64}
    weights::Ptr{Float64}
    derivative_split::Ptr{Float64}
    derivative_dhat::Ptr{Float64}
    inverse_vandermonde_legendre::Ptr{Float64}
    forward_upper::Ptr{Float64}
    forward_lower::Ptr{Float64}
    reverse_upper::Ptr{Float64}
    reverse_lower::Ptr{Float64}
    node_coordinates::Ptr{Float64}
    nghost_elements::Int64
    boundary_neighbor_ids::Ptr{Int64}
    boundary_neighbor_sides::Ptr{Int64}
    boundary_orientations::Ptr{Int64}
    boundary_function::Int32
    source_terms::Int32
    nboundary_params::Int32
    nsource_params::Int32
    boundary_params::NTuple{8, Float64}
    source_params::NTuple{3, Float64}
    nonconservative_flux::Int32
    reserved0::Int32
    glm_speed::Float64
end

flux_code(::typeof(Trixi.flux_ranocha)) = FLUX_RANOCHA
flux_code(::typeof(Trixi.flux_central)) = FLUX_CENTRAL
flux_code(::Trixi.FluxLaxFriedrichs) = FLUX_LAX_FRIEDRICHS
flux_code(::typeof(Trixi.flux_hindenlang_gassner)) = FLUX_HINDENLANG_GASSNER
flux_code(::typeof(Trixi.flux_shima_etal)) = FLUX_SHIMA_ETAL
# flux_hll is FluxHLL(min_max_speed_naive); flux_hlle takes Einfeldt's speeds
flux_code(f::Trixi.FluxHLL) = f.min_max_speed === Trixi.min_max_speed_einfeldt ? FLUX_HLLE : FLUX_HLL
flux_code(::typeof(Trixi.flux_hlle)) = FLUX_HLLE
# equations with nonconservative terms pass (flux, nonconservative_flux) tuples
flux_code(f::Tuple) = flux_code(first(f))
noncons_code(::Any) = NONCONSERVATIVE_NONE
noncons_code(f::Tuple) = last(f) === Trixi.flux_nonconservative_powell ? NONCONSERVATIVE_POWELL : Int32(-1)

function check(status)
    status == 0 && return nothing
    buf = Vector{UInt8}(undef, 1024)
    ccall((:trixi_last_error, libtrixi), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), C_NULL, buf, length(buf))
    error("libtrixi_b200: status $status: " * unsafe_string(pointer(buf)))
end

"""
    create_handle(mesh, equations, solver, cache_cpu; precision = 0)

Builds the library handle from the CPU cache that `SemidiscretizationHyperbolicGPU`
already creates with Trixi's `init_*` (semidiscretization_hyperbolic.jl:69-72):
the connectivity containers are passed as host pointers in their Julia layout,
together with Trixi's own basis matrices (so both sides use identical operators).
"""
function create_handle(mesh, equations, solver, cache_cpu; precision = 0, source_terms = nothing)
    # this glue passes periodic meshes; Dirichlet boundaries go through the
    # descriptor's boundary fields with a built-in boundary function kind
    all(Trixi.isperiodic(mesh)) ||
        error("libtrixi_b200 glue: non-periodic TreeMesh needs the boundaries container and a built-in " *
              "BoundaryConditionDirichlet function kind in the descriptor")
    src = source_code(source_terms)
    elements, interfaces, mortars = cache_cpu.elements, cache_cpu.interfaces, cache_cpu.mortars
    basis = solver.basis
    vi = solver.volume_integral
    vol, vflux, fvflux = VOLUME_WEAK_FORM, FLUX_CENTRAL, FLUX_LAX_FRIEDRICHS
    amax, amin, asmooth, indvar = 0.5, 0.001, Int32(1), Int32(0)
    if vi isa Trixi.VolumeIntegralFluxDifferencing
        vol, vflux = VOLUME_FLUX_DIFFERENCING, flux_code(vi.volume_flux)
    elseif vi isa Trixi.VolumeIntegralShockCapturingHG
        vol, vflux, fvflux = VOLUME_SHOCK_CAPTURING_HG, flux_code(vi.volume_flux_dg), flux_code(vi.volume_flux_fv)
        amax, amin, asmooth = vi.indicator.alpha_max, vi.indicator.alpha_min, Int32(vi.indicator.alpha_smooth)
        indvar = vi.indicator.variable === Trixi.pressure ? Int32(1) : Int32(0)
    end
    eq = equations isa Trixi.AbstractCompressibleEulerEquations ? EQ_COMPRESSIBLE_EULER :
         equations isa Trixi.AbstractIdealGlmMhdEquations ? EQ_IDEAL_GLM_MHD : EQ_LINEAR_ADVECTION
    adv = eq == EQ_LINEAR_ADVECTION ? (Float64.(equations.advection_velocity)..., 0.0, 0.0, 0.0)[1:3] : (0.0, 0.0, 0.0)
    gamma = eq == EQ_LINEAR_ADVECTION ? 1.4 : Float64(equations.gamma)
    # ideal GLM-MHD: the nonconservative flux of the surface pair and c_h
    # (equations.c_h; a GlmSpeedCallback updates it through trixi_set_glm_speed)
    noncons = noncons_code(solver.surface_integral.surface_flux)
    c_h = eq == EQ_IDEAL_GLM_MHD && ndims(mesh) > 1 ? Float64(equations.c_h) : 0.0
    # keep the host arrays alive for the duration of the call
    dsplit = Matrix{Float64}(Array(basis.derivative_split))
    dhat = Matrix{Float64}(Array(basis.derivative_dhat))
    weights = Vector{Float64}(basis.weights)
    # periodic TreeMesh (boundary_function = -1, no source terms); a
    # non-periodic mesh passes cache_cpu.boundaries' neighbor_ids,
    # neighbor_sides and orientations and the Dirichlet function's kind
    desc = ProblemDesc(0, ndims(mesh), Trixi.polydeg(basis), nvariables(equations), eq, vol, vflux,
                       flux_code(solver.surface_integral.surface_flux), fvflux, Int32(precision), gamma, adv,
                       amax, amin, asmooth, indvar,
                       nelements(elements), pointer(elements.inverse_jacobian),
                       ninterfaces(interfaces), pointer(interfaces.neighbor_ids), pointer(interfaces.orientations),
                       0, Trixi.nmortars(mortars), pointer(mortars.neighbor_ids), pointer(mortars.large_sides),
                       pointer(mortars.orientations), pointer(weights), pointer(dsplit), pointer(dhat),
                       C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, pointer(elements.node_coordinates), 0,
                       C_NULL, C_NULL, C_NULL, Int32(-1), src, Int32(0), Int32(0),
                       ntuple(_ -> 0.0, 8), ntuple(_ -> 0.0, 3), noncons, Int32(0), c_h)
    desc.struct_size = Int32(sizeof(ProblemDesc))
    handle = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve elements interfaces mortars dsplit dhat weights desc begin
        check(ccall((:trixi_create, libtrixi), Cint, (Ref{ProblemDesc}, Ref{Ptr{Cvoid}}), desc, handle))
    end
    h = handle[]
    return h
end

stream_ptr() = reinterpret(Ptr{Cvoid}, CUDA.stream().handle)

# rhs_gpu!(du_ode, u_ode, semi, t) -- src/solvers/solvers.jl:18-31
function rhs_gpu!(du_ode::CuArray{Float64}, u_ode::CuArray{Float64}, handle::Ptr{Cvoid}, t)
    check(ccall((:trixi_rhs, libtrixi), Cint, (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Float64, Ptr{Cvoid}),
                handle, pointer(du_ode), pointer(u_ode), Float64(t), stream_ptr()))
    return nothing
end

# one fused CarpenterKennedy2N54 stage: k <- a k + dt rhs(u_in); u_out <- u_in + b k
function rk_stage!(u_out, u_in, k, a, b, dt, t, handle)
    check(ccall((:trixi_rk_stage, libtrixi), Cint,
                (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Float64, Float64, Float64, Float64, Ptr{Cvoid}),
                handle, pointer(u_out), pointer(u_in), pointer(k), a, b, dt, t, stream_ptr()))
end

# stage functions of the reference (cuda_volume_integral!, ...), e.g.
cuda_volume_integral!(du, u, handle) =
    check(ccall((:trixi_volume_integral, libtrixi), Cint, (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Ptr{Cvoid}),
                handle, pointer(du), pointer(u), stream_ptr()))
cuda_prolong2interfaces!(u, handle) =
    check(ccall((:trixi_prolong2interfaces, libtrixi), Cint, (Ptr{Cvoid}, CuPtr{Float64}, Ptr{Cvoid}),
                handle, pointer(u), stream_ptr()))
cuda_interface_flux!(handle) =
    check(ccall((:trixi_interface_flux, libtrixi), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), handle, stream_ptr()))
cuda_surface_integral!(du, handle) =
    check(ccall((:trixi_surface_integral, libtrixi), Cint, (Ptr{Cvoid}, CuPtr{Float64}, Ptr{Cvoid}),
                handle, pointer(du), stream_ptr()))
cuda_jacobian!(du, handle) =
    check(ccall((:trixi_jacobian, libtrixi), Cint, (Ptr{Cvoid}, CuPtr{Float64}, Ptr{Cvoid}),
                handle, pointer(du), stream_ptr()))

# ---- discrete adjoint as ChainRulesCore rules --------------------------------
# The Julia counterpart of trixicuda/adjoint.py's torch.autograd.Functions:
# Zygote (or any ChainRules-aware AD) differentiates through the library's
# hand-written reverse kernels instead of tracing Julia code.

"du = rhs(u): one fused rhs evaluation (t = 0)."
function rhs(u::CuArray{Float64}, handle::Ptr{Cvoid})
    du = similar(u)
    rhs_gpu!(du, u, handle, 0.0)
    return du
end

function ChainRulesCore.rrule(::typeof(rhs), u::CuArray{Float64}, handle::Ptr{Cvoid})
    du = rhs(u, handle)
    function rhs_pullback(dū)
        λ = CuArray{Float64}(unthunk(dū))
        ū = similar(u)
        check(ccall((:trixi_rhs_vjp, libtrixi), Cint,
                    (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Ptr{Cvoid}),
                    handle, pointer(ū), pointer(u), pointer(λ), stream_ptr()))
        return NoTangent(), ū, NoTangent()
    end
    return du, rhs_pullback
end

"uT = ck2n54(u0, dt, nsteps, nsnapshots, handle): nsteps CarpenterKennedy2N54 steps."
function ck2n54(u0::CuArray{Float64}, dt, nsteps, nsnapshots, handle::Ptr{Cvoid})
    uT = similar(u0)
    check(ccall((:trixi_adjoint_forward, libtrixi), Cint,
                (Ptr{Cvoid}, CuPtr{Float64}, Float64, Int64, Int64, CuPtr{Float64}, Ptr{Cvoid}),
                handle, pointer(u0), Float64(dt), Int64(nsteps), Int64(nsnapshots), pointer(uT), stream_ptr()))
    return uT
end

# reverse sweep over the stored (binomial) checkpoints, recomputing the rest
function ChainRulesCore.rrule(::typeof(ck2n54), u0::CuArray{Float64}, dt, nsteps, nsnapshots, handle::Ptr{Cvoid})
    uT = ck2n54(u0, dt, nsteps, nsnapshots, handle)
    function ck2n54_pullback(ūT)
        g = CuArray{Float64}(unthunk(ūT))
        ū0 = similar(u0)
        recomputed = Ref{Int64}(0)
        check(ccall((:trixi_adjoint_backward, libtrixi), Cint,
                    (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Ref{Int64}, Ptr{Cvoid}),
                    handle, pointer(g), pointer(ū0), recomputed, stream_ptr()))
        return NoTangent(), ū0, NoTangent(), NoTangent(), NoTangent(), NoTangent()
    end
    return uT, ck2n54_pullback
end

# GlmSpeedCallback: equations.c_h changed between steps
set_glm_speed!(handle, c_h) =
    check(ccall((:trixi_set_glm_speed, libtrixi), Cint, (Ptr{Cvoid}, Float64), handle, Float64(c_h)))

destroy!(handle) = ccall((:trixi_destroy, libtrixi), Cint, (Ptr{Cvoid},), handle)

end # module
