# BEMGPU.jl -- drop-in full-3D BEM for AcousticScattering.jl on one GB300 through ccall.
#
# Adds a BEMSolution payload type, `_GPUBEMData`, and methods of the reference's own
# generic functions (`scattering_amplitude`, `target_strength`, `diagnostics`) for it;
# `BEMGPU.bem(surface, boundary, k; ...)` replaces `bem(surface::Mesh, boundary, k; ...)`
# (solvers/bem/surface.jl:10-23 of AcousticScattering.jl) for supplied flat-triangle
# surfaces.  Every numerical step runs in libbemgpu.so (C ABI: include/bemgpu.h).
#
# Julia is not installed where this library is built and tested; this module is the
# binding a maintainer adds on the Julia side (the Python mirror in ../bemgpu/ is the
# tested host of the same C ABI).
module BEMGPU

using LinearAlgebra
import AcousticScattering
import AcousticScattering: bem, scattering_amplitude, target_strength, diagnostics, pressure,
    BEMSolution, Rigid, PressureRelease, FluidFilled, Mesh, incidence_angle_sweep,
    frequency_sweep, IncidenceAngleSweep, FrequencySweep

const libbemgpu = joinpath(@__DIR__, "..", "bemgpu", "libbemgpu.so")

const OK, EINVAL, ETOPOLOGY = 0, 1, 2
const ENOTCONVERGED = 5

struct Problem
    boundary::Int32
    formulation::Int32
    precision::Int32
    equilibrate::Int32
    k::Float64
    density_contrast::Float64
    soundspeed_contrast::Float64
    refine_tolerance::Float64
    refine_maxiter::Int32
    assembly::Int32
    condition_guard::Float64
    near_eta::Float64
    discretization::Int32   # 0 collocation, 1 Nyström (the reference's correction=(method=:dim,))
    condition_limit::Int32  # SVD condition numbers up to this order (full.jl:364-409)
    norm_floor::Float64     # lower bound of the equilibration scales (double precision)
end

struct Diagnostics
    unknown_count::Int64
    quadrature_nodes::Int64
    near_pairs::Int64
    formulation::Int32
    precision::Int32
    factor_precision::Int32
    refinement_reason::Int32
    refinement_iterations::Int32
    equilibrate::Int32
    coupling_re::Float64
    coupling_im::Float64
    absolute_residual::Float64
    relative_residual::Float64
    scaled_absolute_residual::Float64
    scaled_relative_residual::Float64
    normwise_backward_error::Float64
    componentwise_backward_error::Float64
    single_reciprocal_condition::Float64
    assemble_ms::Float64
    factor_ms::Float64
    solve_ms::Float64
    total_ms::Float64
    device_bytes::Int64
    nrhs::Int32
    info::Int32
    condition_number::Float64
    scaled_condition_number::Float64
    conditioning::Int32
    condition_limit::Int32
    derivative_exterior::Int32
    derivative_interior::Int32
end

function last_error(ctx)
    buf = Vector{UInt8}(undef, 512)
    ccall((:bemgpu_last_error, libbemgpu), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t),
        ctx, buf, length(buf))
    return unsafe_string(pointer(buf))
end

function check(status, ctx = C_NULL)
    status == OK && return nothing
    msg = last_error(ctx)
    status in (EINVAL, ETOPOLOGY) && throw(ArgumentError(msg))
    status == ENOTCONVERGED && error(msg)
    error("libbemgpu: " * msg)
end

mutable struct Context
    ptr::Ptr{Cvoid}
    function Context(device::Integer = 0; hbm_budget::Integer = 0)
        r = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:bemgpu_ctx_create, libbemgpu), Cint, (Cint, UInt64, Ptr{Ptr{Cvoid}}),
            device, hbm_budget, r))
        c = new(r[])
        finalizer(x -> ccall((:bemgpu_ctx_destroy, libbemgpu), Cint, (Ptr{Cvoid},), x.ptr), c)
        return c
    end
end

const DEFAULT = Ref{Union{Nothing, Context}}(nothing)
context() = (DEFAULT[] === nothing && (DEFAULT[] = Context()); DEFAULT[])

mutable struct GPUMesh
    ptr::Ptr{Cvoid}
    nodes::Matrix{Float64}
    triangles::Matrix{Int64}
end

"""
    upload(ctx, nodes::3xN, triangles::3xM) -> GPUMesh

Validates the surface exactly as `mesh(nodes, triangles)` does (geometry/surface.jl:341-405)
and uploads it.
"""
function upload(ctx::Context, nodes::AbstractMatrix{<:Real}, triangles::AbstractMatrix{<:Integer})
    n = Matrix{Float64}(nodes)
    t = Matrix{Int64}(triangles)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bemgpu_mesh_upload, libbemgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Int64, Ptr{Int64}, Int64, Ptr{Ptr{Cvoid}}),
        ctx.ptr, n, size(n, 2), t, size(t, 2), r), ctx.ptr)
    m = GPUMesh(r[], n, t)
    finalizer(x -> ccall((:bemgpu_mesh_destroy, libbemgpu), Cint, (Ptr{Cvoid},), x.ptr), m)
    return m
end

"""
    upload(ctx, surface::AcousticScattering.Mesh) -> GPUMesh

The nodes and flat triangles of a surface built by the reference's `mesh(nodes,
triangles)` (geometry/surface.jl:271-298; its `_SurfaceGeometry` body keeps the supplied
nodes in meters and one corner list per triangle), validated and uploaded.
"""
function upload(ctx::Context, surface::Mesh)
    geom = surface.body
    geom isa AcousticScattering._SurfaceGeometry || throw(ArgumentError(
        "BEMGPU solves supplied triangle surfaces (mesh(nodes, triangles)); mesh generated " *
        "bodies with mesh(nodes, triangles) first"))
    all(c -> length(c) == 3, geom.connectivity) ||
        throw(ArgumentError("BEMGPU needs flat three-node triangles"))
    tris = Matrix{Int64}(undef, 3, length(geom.connectivity))
    for (j, c) in enumerate(geom.connectivity)
        tris[:, j] .= c
    end
    return upload(ctx, geom.nodes, tris)
end

struct _GPUBEMData
    solution::Ptr{Cvoid}
    nodes::Matrix{Float64}
    triangles::Matrix{Int64}
    incidence_angle::Float64
    incidence_azimuth::Float64
    diagnostics::Diagnostics
    compressed::Bool        # compressed operators + GMRES (its diagnostics add GMRES's)
end
_GPUBEMData(sol, nodes, triangles, angle, azimuth, d) =
    _GPUBEMData(sol, nodes, triangles, angle, azimuth, d, false)

# the reference's `_FullBEMSurfaceData` fields p_scat and dpdn_scat (types.jl:2-11): the
# scattered traces at every unknown location, read from the device when asked for
function Base.getproperty(d::_GPUBEMData, name::Symbol)
    if name === :p_scat || name === :dpdn_scat
        n = Int(getfield(d, :diagnostics).quadrature_nodes)
        p = zeros(Float64, 2n)
        q = zeros(Float64, 2n)
        check(ccall((:bemgpu_traces, libbemgpu), Cint,
            (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}), getfield(d, :solution), 0, p, q))
        v = name === :p_scat ? p : q
        return [complex(v[2i - 1], v[2i]) for i in 1:n]
    end
    return getfield(d, name)
end

_boundary_code(::Rigid) = Int32(0)
_boundary_code(::PressureRelease) = Int32(1)
_boundary_code(::FluidFilled) = Int32(2)
const FORMULATIONS = Dict(:burton_miller => Int32(0), :cbie => Int32(1), :muller => Int32(2))

struct HmatrixOptions
    tol::Float64
    eta::Float64
    leaf_size::Int32
    restart::Int32
    reltol::Float64
    abstol::Float64
    maxiter::Int32
    neighbours::Int32       # Schwarz neighbourhood of Nyström rigid systems (0 = none)
end

struct HmatrixStats
    lowrank_blocks::Int64
    dense_blocks::Int64
    densified_blocks::Int64
    lowrank_entries::Int64
    dense_entries::Int64
    max_rank::Int32
    depth::Int32
    leaves::Int32
    pad::Int32
    compression::Float64
    gmres_iterations::Int32
    gmres_converged::Int32
    build_ms::Float64
    gmres_ms::Float64
end

"""
    bem(gpu_mesh, boundary, k; incidence_angle=π/2, incidence_azimuth=0, formulation,
        precision=:double, equilibrate=true, refinement=(;), assembly=:default,
        compression=(method=:none,), gmres_kwargs=(;))

The reference's `bem(surface::Mesh, boundary, k; ...)` on the GPU.  With
`compression=(method=:hmatrix, tol=1e-5)` a Rigid or PressureRelease body is solved as the
reference's `solve_full_bem` does by default: compressed operators and GMRES with
`gmres_kwargs` (reltol, abstol, restart, maxiter); non-convergence warns as there.
`discretization=:nystrom` solves on the quadrature nodes with the density-interpolation
correction, as the reference's default `correction=(method=:dim,)` does (dense factor, or
with `compression` the compressed node operators and GMRES for Rigid/PressureRelease).
"""
function bem(m::GPUMesh, boundary, k::Real; incidence_angle::Real = π / 2,
        incidence_azimuth::Real = 0.0, formulation::Union{Nothing, Symbol} = nothing,
        precision::Symbol = :double, equilibrate::Bool = true,
        refinement::NamedTuple = (;), assembly::Symbol = :default,
        compression::NamedTuple = (method = :none,), gmres_kwargs::NamedTuple = (;),
        discretization::Symbol = :collocation, condition_limit::Integer = 512,
        norm_floor::Real = 0.0, ctx::Context = context())
    isfinite(k) && k > 0 || throw(ArgumentError("k must be finite and positive"))
    discretization in (:collocation, :nystrom) ||
        throw(ArgumentError("discretization must be :collocation or :nystrom"))
    method = get(compression, :method, :none)
    method in (:none, :hmatrix) ||
        throw(ArgumentError("compression method must be :none or :hmatrix"))
    if method === :hmatrix
        boundary isa FluidFilled && throw(ArgumentError(
            "hierarchical compression applies to Rigid and PressureRelease boundaries"))
        p = Problem(_boundary_code(boundary),
            formulation === nothing ? Int32(-1) : FORMULATIONS[formulation],
            precision === :mixed ? Int32(1) : Int32(0), Int32(1), Float64(k), 1.0, 1.0,
            1e-13, Int32(8), Int32(0), 10eps(Float32), 2.0,
            discretization === :nystrom ? Int32(1) : Int32(0), Int32(condition_limit),
        Float64(norm_floor))
        o = HmatrixOptions(get(compression, :tol, 1e-5), get(compression, :eta, 3.0),
            Int32(get(compression, :leaf_size, 64)), Int32(get(gmres_kwargs, :restart, 150)),
            get(gmres_kwargs, :reltol, 1e-4), get(gmres_kwargs, :abstol, 0.0),
            Int32(get(gmres_kwargs, :maxiter, 1200)), Int32(get(compression, :neighbours, 0)))
        inc = Float64[incidence_angle, incidence_azimuth]
        r = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:bemgpu_hmatrix_solve, libbemgpu), Cint,
            (Ptr{Cvoid}, Ptr{Cvoid}, Ref{Problem}, Ref{HmatrixOptions}, Int32, Ptr{Float64},
                Ptr{Ptr{Cvoid}}),
            ctx.ptr, m.ptr, p, o, 1, inc, r), ctx.ptr)
        st = Ref{HmatrixStats}()
        ccall((:bemgpu_hmatrix_stats_get, libbemgpu), Cint, (Ptr{Cvoid}, Ref{HmatrixStats}),
            r[], st)
        st[].gmres_converged == 1 ||
            @warn "solve_full_bem: GMRES did not converge to the requested tolerance, result may be inaccurate" boundary iters = st[].gmres_iterations
        d = Ref{Diagnostics}()
        ccall((:bemgpu_solution_diagnostics, libbemgpu), Cint, (Ptr{Cvoid}, Ref{Diagnostics}),
            r[], d)
        data = _GPUBEMData(r[], m.nodes, m.triangles, incidence_angle, incidence_azimuth, d[],
            true)
        return BEMSolution(AcousticScattering._SurfaceGeometry(m.nodes, m.triangles), boundary,
            Float64(k), :full, data)
    end
    g, h = boundary isa FluidFilled ?
           (boundary.density_contrast, boundary.soundspeed_contrast) : (1.0, 1.0)
    p = Problem(_boundary_code(boundary),
        formulation === nothing ? Int32(-1) : FORMULATIONS[formulation],
        precision === :mixed ? Int32(1) : Int32(0), Int32(equilibrate), Float64(k), g, h,
        get(refinement, :tolerance, 1e-13), Int32(get(refinement, :maxiter, 8)),
        assembly === :double ? Int32(1) : assembly === :single ? Int32(2) : Int32(0),
        get(refinement, :condition_guard, 10eps(Float32)), 2.0,
        discretization === :nystrom ? Int32(1) : Int32(0), Int32(condition_limit),
        Float64(norm_floor))
    inc = Float64[incidence_angle, incidence_azimuth]
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bemgpu_solve, libbemgpu), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ref{Problem}, Int32, Ptr{Float64}, Ptr{Ptr{Cvoid}}),
        ctx.ptr, m.ptr, p, 1, inc, r), ctx.ptr)
    d = Ref{Diagnostics}()
    ccall((:bemgpu_solution_diagnostics, libbemgpu), Cint, (Ptr{Cvoid}, Ref{Diagnostics}), r[], d)
    data = _GPUBEMData(r[], m.nodes, m.triangles, incidence_angle, incidence_azimuth, d[])
    return BEMSolution(AcousticScattering._SurfaceGeometry(m.nodes, m.triangles), boundary,
        Float64(k), :full, data)
end

"""
    bem(surface::AcousticScattering.Mesh, boundary, k; kwargs...)

The reference's own entry point, `bem(surface::Mesh, boundary, k; ...)`
(solvers/bem/surface.jl:10-23), for a surface from `mesh(nodes, triangles)`: the surface
is uploaded (`upload(ctx, surface)`) and solved as `bem(gpu_mesh, boundary, k; ...)`.
"""
bem(surface::Mesh, boundary::Union{Rigid, PressureRelease, FluidFilled}, k::Real;
    ctx::Context = context(), kwargs...) = bem(upload(ctx, surface), boundary, k; ctx, kwargs...)

function _problem(boundary, k; formulation = nothing, precision = :double,
        equilibrate = true, refinement = (;), assembly = :default,
        discretization = :collocation, condition_limit = 512, norm_floor = 0.0)
    g, h = boundary isa FluidFilled ?
           (boundary.density_contrast, boundary.soundspeed_contrast) : (1.0, 1.0)
    return Problem(_boundary_code(boundary),
        formulation === nothing ? Int32(-1) : FORMULATIONS[formulation],
        precision === :mixed ? Int32(1) : Int32(0), Int32(equilibrate), Float64(k), g, h,
        get(refinement, :tolerance, 1e-13), Int32(get(refinement, :maxiter, 8)),
        assembly === :double ? Int32(1) : assembly === :single ? Int32(2) : Int32(0),
        get(refinement, :condition_guard, 10eps(Float32)), 2.0,
        discretization === :nystrom ? Int32(1) : Int32(0), Int32(condition_limit),
        Float64(norm_floor))
end

function _backscatter(solution::Ptr{Cvoid}, nrhs::Integer)
    out = zeros(Float64, 2)
    amps = Vector{ComplexF64}(undef, nrhs)
    for r in 1:nrhs
        check(ccall((:bemgpu_far_field, libbemgpu), Cint,
            (Ptr{Cvoid}, Int32, Int64, Ptr{Float64}, Ptr{Float64}),
            solution, r - 1, 1, C_NULL, out))
        amps[r] = complex(out[1], out[2])
    end
    return amps
end

"""
    incidence_angle_sweep(gpu_mesh | surface::Mesh, boundary, k, angles;
        incidence_azimuth=0, formulation, precision=:double, equilibrate=true,
        refinement=(;), assembly=:default, discretization=:collocation)

The reference's dense-factor `incidence_angle_sweep` (postprocessing/sweeps.jl:626-701):
assembled and factored once, every polar angle (radians from +x) solved as one
multi-right-hand-side batch; backscatter amplitudes and target strengths in the
reference's `IncidenceAngleSweep`.
"""
function incidence_angle_sweep(m::GPUMesh, boundary::Union{Rigid, PressureRelease, FluidFilled},
        k::Real, angles::AbstractVector{<:Real}; incidence_azimuth::Real = 0.0,
        ctx::Context = context(), kwargs...)
    isempty(angles) && throw(ArgumentError("a sweep needs at least one sample"))
    all(isfinite, angles) || throw(ArgumentError("sweep coordinates must be finite"))
    isfinite(incidence_azimuth) || throw(ArgumentError("incidence azimuth must be finite"))
    p = _problem(boundary, k; kwargs...)
    f = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bemgpu_factor_create, libbemgpu), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ref{Problem}, Ptr{Ptr{Cvoid}}), ctx.ptr, m.ptr, p, f), ctx.ptr)
    try
        inc = Float64[x for a in angles for x in (Float64(a), Float64(incidence_azimuth))]
        r = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:bemgpu_factor_solve, libbemgpu), Cint,
            (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Ptr{Cvoid}}), f[], length(angles), inc, r),
            ctx.ptr)
        amps = try
            _backscatter(r[], length(angles))
        finally
            ccall((:bemgpu_solution_destroy, libbemgpu), Cint, (Ptr{Cvoid},), r[])
        end
        return IncidenceAngleSweep(Float64.(angles), 20 .* log10.(abs.(amps)), amps, String[])
    finally
        ccall((:bemgpu_factor_destroy, libbemgpu), Cint, (Ptr{Cvoid},), f[])
    end
end

incidence_angle_sweep(surface::Mesh, boundary::Union{Rigid, PressureRelease, FluidFilled},
    k::Real, angles::AbstractVector{<:Real}; ctx::Context = context(), kwargs...) =
    incidence_angle_sweep(upload(ctx, surface), boundary, k, angles; ctx, kwargs...)

"""
    frequency_sweep(gpu_mesh | surface::Mesh, boundary, frequencies, sound_speed;
        incidence_angle=π/2, incidence_azimuth=0, kwargs...)

Backscatter over frequencies (postprocessing/sweeps.jl:103-110 computes the same
`FrequencySweep` by calling `bem` once per frequency): every frequency's system is
assembled, factored and solved in one batched launch sequence.
"""
function frequency_sweep(m::GPUMesh, boundary::Union{Rigid, PressureRelease, FluidFilled},
        frequencies::AbstractVector{<:Real}, sound_speed::Real;
        incidence_angle::Real = π / 2, incidence_azimuth::Real = 0.0,
        ctx::Context = context(), kwargs...)
    isfinite(sound_speed) && sound_speed > 0 ||
        throw(ArgumentError("sound_speed must be finite and positive"))
    all(>(0), frequencies) || throw(ArgumentError("frequencies must be positive"))
    ks = 2π .* Float64.(frequencies) ./ Float64(sound_speed)
    count = length(ks)
    probs = [_problem(boundary, k; kwargs...) for k in ks]
    meshes = fill(m.ptr, count)
    factors = fill(C_NULL, count)
    check(ccall((:bemgpu_factor_create_batch, libbemgpu), Cint,
        (Ptr{Cvoid}, Int32, Ptr{Ptr{Cvoid}}, Ptr{Problem}, Ptr{Ptr{Cvoid}}),
        ctx.ptr, count, meshes, probs, factors), ctx.ptr)
    sols = fill(C_NULL, count)
    try
        nrhs = fill(Int32(1), count)
        inc = [Float64[incidence_angle, incidence_azimuth] for _ in 1:count]
        incp = [pointer(v) for v in inc]
        GC.@preserve inc check(ccall((:bemgpu_factor_solve_batch, libbemgpu), Cint,
            (Ptr{Cvoid}, Int32, Ptr{Ptr{Cvoid}}, Ptr{Int32}, Ptr{Ptr{Float64}},
                Ptr{Ptr{Cvoid}}), ctx.ptr, count, factors, nrhs, incp, sols), ctx.ptr)
        amps = [_backscatter(s, 1)[1] for s in sols]
        return FrequencySweep(Float64.(frequencies), ks, 20 .* log10.(abs.(amps)), amps,
            String[])
    finally
        for s in sols
            s == C_NULL || ccall((:bemgpu_solution_destroy, libbemgpu), Cint, (Ptr{Cvoid},), s)
        end
        for f in factors
            f == C_NULL || ccall((:bemgpu_factor_destroy, libbemgpu), Cint, (Ptr{Cvoid},), f)
        end
    end
end

frequency_sweep(surface::Mesh, boundary::Union{Rigid, PressureRelease, FluidFilled},
    frequencies::AbstractVector{<:Real}, sound_speed::Real; ctx::Context = context(),
    kwargs...) = frequency_sweep(upload(ctx, surface), boundary, frequencies, sound_speed;
    ctx, kwargs...)

"""
    bem(gpu_meshes::Vector{GPUMesh}, materials::Vector{FluidFilled}, k;
        parents=collect(0:length(gpu_meshes)-1), incidence_angle=π/2, incidence_azimuth=0,
        formulation=:muller, precision=:double, equilibrate=true, refinement=(;))

The reference's coupled-region `bem(surfaces, materials, k; parents, ...)`
(solvers/bem/regions.jl:132-150) on the GPU.  The returned solution answers
`scattering_amplitude` / `target_strength` (summed over the surfaces bordering the
exterior, solvers/bem/postprocessing.jl:15-31) and `diagnostics`.
"""
function bem(ms::AbstractVector{GPUMesh}, materials::AbstractVector{<:FluidFilled}, k::Real;
        parents::AbstractVector{<:Integer} = collect(0:(length(ms) - 1)),
        incidence_angle::Real = π / 2, incidence_azimuth::Real = 0.0,
        formulation::Symbol = :muller, precision::Symbol = :double, equilibrate::Bool = true,
        refinement::NamedTuple = (;), assembly::Symbol = :default,
        condition_limit::Integer = 512, ctx::Context = context())
    count = length(ms)
    length(materials) == length(parents) == count ||
        throw(ArgumentError("supply one material and parent per interface"))
    p = Problem(Int32(2), FORMULATIONS[formulation],
        precision === :mixed ? Int32(1) : Int32(0), Int32(equilibrate), Float64(k), 1.0, 1.0,
        get(refinement, :tolerance, 1e-13), Int32(get(refinement, :maxiter, 8)),
        assembly === :double ? Int32(1) : assembly === :single ? Int32(2) : Int32(0),
        get(refinement, :condition_guard, 10eps(Float32)), 2.0, Int32(0),
        Int32(condition_limit), 0.0)
    handles = Ptr{Cvoid}[m.ptr for m in ms]
    dens = Float64[m.density_contrast for m in materials]
    speeds = Float64[m.soundspeed_contrast for m in materials]
    par = Int32.(parents)
    inc = Float64[incidence_angle, incidence_azimuth]
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bemgpu_region_solve, libbemgpu), Cint,
        (Ptr{Cvoid}, Int32, Ptr{Ptr{Cvoid}}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32},
            Ref{Problem}, Int32, Ptr{Float64}, Ptr{Ptr{Cvoid}}),
        ctx.ptr, count, handles, dens, speeds, par, p, 1, inc, r), ctx.ptr)
    d = Ref{Diagnostics}()
    ccall((:bemgpu_solution_diagnostics, libbemgpu), Cint, (Ptr{Cvoid}, Ref{Diagnostics}), r[], d)
    data = _GPUBEMData(r[], ms[1].nodes, ms[1].triangles, incidence_angle, incidence_azimuth,
        d[])
    return BEMSolution(AcousticScattering._SurfaceGeometry(ms[1].nodes, ms[1].triangles),
        materials[1], Float64(k), :full, data)
end

function scattering_amplitude(sol::BEMSolution{_GPUBEMData};
        direction::Union{Nothing, AbstractVector} = nothing)
    out = zeros(Float64, 2)
    if direction === nothing
        check(ccall((:bemgpu_far_field, libbemgpu), Cint,
            (Ptr{Cvoid}, Int32, Int64, Ptr{Float64}, Ptr{Float64}),
            sol.data.solution, 0, 1, C_NULL, out))
    else
        d = Float64.(collect(direction))
        check(ccall((:bemgpu_far_field, libbemgpu), Cint,
            (Ptr{Cvoid}, Int32, Int64, Ptr{Float64}, Ptr{Float64}),
            sol.data.solution, 0, 1, d, out))
    end
    return complex(out[1], out[2])
end

const FIELDS = Dict(:total => Int32(0), :scattered => Int32(1), :incident => Int32(2),
    :interior => Int32(3))

"""
    pressure(sol::BEMSolution{_GPUBEMData}, points; field=:total, region=nothing)

The reference's `pressure(solution, points; field, region)` (fields/pressure.jl:42-53;
coupled regions fields/regions.jl:1-65): one point (3 numbers) gives a complex value, a
vector of points a vector.
"""
function pressure(sol::BEMSolution{_GPUBEMData}, points; field::Symbol = :total,
        region::Union{Nothing, Integer} = nothing)
    haskey(FIELDS, field) ||
        throw(ArgumentError("field must be :total, :scattered, :incident or :interior"))
    single = points isa AbstractVector{<:Real}
    pts = single ? [points] : collect(points)
    flat = Float64[c for p in pts for c in p]
    length(flat) == 3 * length(pts) || throw(ArgumentError("a point has three coordinates"))
    out = zeros(Float64, 2 * length(pts))
    check(ccall((:bemgpu_pressure_region, libbemgpu), Cint,
        (Ptr{Cvoid}, Int32, Int64, Ptr{Float64}, Int32, Int32, Ptr{Float64}),
        sol.data.solution, 0, length(pts), flat, FIELDS[field],
        region === nothing ? Int32(-1) : Int32(region), out))
    values = [complex(out[2i - 1], out[2i]) for i in 1:length(pts)]
    return single ? values[1] : values
end

# ------------------------------------------------------------------ serving
struct ServerOptions
    max_batch::Int32
    queue_limit::Int32
    cache_bytes::UInt64
    lanes::Int32
    reserved::Int32
end

struct ServerStats
    submitted::Int64
    completed::Int64
    failed::Int64
    items::Int64
    factorizations::Int64
    cache_hits::Int64
    batches::Int64
    evictions::Int64
    busy_ms::Float64
    cached_bytes::UInt64
    retries::Int64
end

"""
    Server(ctx=context(); max_batch=64, queue_limit=4096, cache_bytes=0, lanes=2)

The library's continuous-batching request loop (no reference counterpart): `submit`
queues one surface / boundary problem at several wavenumbers and incidence directions and
returns a ticket, `wait` returns its backscatter amplitudes (nfreq × nangles) and latency
in ms.  `lanes` batches run on the device at once; factors are cached across requests.
"""
mutable struct Server
    ptr::Ptr{Cvoid}
    ctx::Context
    shapes::Dict{Int64, Tuple{Int, Int}}
    function Server(ctx::Context = context(); max_batch::Integer = 64,
            queue_limit::Integer = 4096, cache_bytes::Integer = 0, lanes::Integer = 2)
        o = ServerOptions(Int32(max_batch), Int32(queue_limit), UInt64(cache_bytes),
            Int32(lanes), Int32(0))
        r = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:bemgpu_server_create, libbemgpu), Cint,
            (Ptr{Cvoid}, Ref{ServerOptions}, Ptr{Ptr{Cvoid}}), ctx.ptr, o, r), ctx.ptr)
        s = new(r[], ctx, Dict{Int64, Tuple{Int, Int}}())
        finalizer(close, s)
        return s
    end
end

function submit(s::Server, m::GPUMesh, boundary, ks::AbstractVector{<:Real},
        angles::AbstractVector{<:Real}; azimuth::Real = 0.0, kwargs...)
    isempty(ks) && throw(ArgumentError("at least one wavenumber"))
    p = _problem(boundary, ks[1]; kwargs...)
    inc = Float64[v for a in angles for v in (Float64(a), Float64(azimuth))]
    t = Ref{Int64}(0)
    check(ccall((:bemgpu_server_submit, libbemgpu), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ref{Problem}, Int32, Ptr{Float64}, Int32, Ptr{Float64},
            Ptr{Int64}),
        s.ptr, m.ptr, p, length(ks), Float64.(collect(ks)), length(angles), inc, t), s.ctx.ptr)
    s.shapes[t[]] = (length(ks), length(angles))
    return t[]
end

function Base.wait(s::Server, ticket::Integer; timeout_ms::Integer = -1)
    nf, na = s.shapes[ticket]
    out = zeros(Float64, 2 * nf * na)
    lat = Ref{Float64}(0.0)
    st = ccall((:bemgpu_server_wait, libbemgpu), Cint,
        (Ptr{Cvoid}, Int64, Int32, Ptr{Float64}, Ptr{Float64}),
        s.ptr, ticket, Int32(timeout_ms), out, lat)
    st == 6 && error("request not finished")  # BEMGPU_ETIMEOUT: the ticket stays valid
    delete!(s.shapes, ticket)
    check(st, s.ctx.ptr)
    amps = [complex(out[2q - 1], out[2q]) for q in 1:(nf * na)]
    return permutedims(reshape(amps, na, nf)), lat[]   # nfreq × nangles
end

function stats(s::Server)
    st = Ref{ServerStats}()
    check(ccall((:bemgpu_server_stats_get, libbemgpu), Cint, (Ptr{Cvoid}, Ref{ServerStats}),
        s.ptr, st), s.ctx.ptr)
    return st[]
end

function Base.close(s::Server)
    if s.ptr != C_NULL
        ccall((:bemgpu_server_destroy, libbemgpu), Cint, (Ptr{Cvoid},), s.ptr)
        s.ptr = C_NULL
    end
    return nothing
end

target_strength(sol::BEMSolution{_GPUBEMData}; kwargs...) =
    20 * log10(abs(scattering_amplitude(sol; kwargs...)))

"""
    residual_history(sol) -> Vector{Float64}

GMRES residual estimates, one per Arnoldi step, of a compressed-operator solution (the
reference's `residual_history` diagnostic, full.jl:160-176).
"""
function residual_history(sol::BEMSolution{_GPUBEMData})
    cnt = Ref{Int32}(0)
    check(ccall((:bemgpu_gmres_history, libbemgpu), Cint,
        (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32, Ptr{Int32}),
        sol.data.solution, 0, C_NULL, 0, cnt))
    out = zeros(Float64, max(1, cnt[]))
    check(ccall((:bemgpu_gmres_history, libbemgpu), Cint,
        (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32, Ptr{Int32}),
        sol.data.solution, 0, out, length(out), cnt))
    return out[1:cnt[]]
end

function diagnostics(sol::BEMSolution{_GPUBEMData})
    if sol.data.compressed  # the reference's GMRES diagnostics (full.jl:160-176)
        st = Ref{HmatrixStats}()
        check(ccall((:bemgpu_hmatrix_stats_get, libbemgpu), Cint,
            (Ptr{Cvoid}, Ref{HmatrixStats}), sol.data.solution, st))
        return merge(_diagnostics(sol.data.diagnostics), (; method = :gmres,
            converged = st[].gmres_converged == 1, iterations = Int(st[].gmres_iterations),
            residual_history = residual_history(sol), compression = st[]))
    end
    return _diagnostics(sol.data.diagnostics)
end

function _diagnostics(d::Diagnostics)
    reasons = (:none, :conversion, :single_singular, :condition, :nonfinite,
        :iteration_limit, :stagnation)
    return (; unknown_count = d.unknown_count, quadrature_nodes = d.quadrature_nodes,
        relative_residual = d.relative_residual, absolute_residual = d.absolute_residual,
        scaled_relative_residual = d.scaled_relative_residual,
        factor_precision = d.factor_precision == 0 ? :single : :double,
        refinement_reason = reasons[d.refinement_reason + 1],
        refinement_iterations = d.refinement_iterations,
        normwise_backward_error = d.normwise_backward_error,
        componentwise_backward_error = d.componentwise_backward_error,
        coupling = complex(d.coupling_re, d.coupling_im), method = d.precision == 1 ?
                                                                    :mixed_refinement : :direct,
        equilibrate = d.equilibrate == 1, condition_limit = d.condition_limit,
        conditioning = d.conditioning == 1 ? :svd : :not_computed,
        condition_number = d.conditioning == 1 ? d.condition_number : nothing,
        scaled_condition_number = d.conditioning == 1 ? d.scaled_condition_number : nothing,
        derivative_evaluation = d.derivative_exterior == 0 ? nothing :
                                (exterior = :direct, interior = :direct))
end

end # module
