"""
    MCRTGB300

Julia binding of libmcrt for MonteCarloRadiativeTransfer.jl: `MCRTGB300.simulate(cfg, g, I₀)`
returns what the package's `simulate(cfg, g, I₀; use_gpu=true)` returns
(src/MonteCarloRadiativeTransfer.jl:26-85), and `MCRTGB300.run_rt(cfg, g)` what its
`run_rt(cfg, g; use_gpu=true)` returns (:87-291), computed by libmcrt's CUDA kernels.

The library path defaults to the in-tree build and can be overridden with the
environment variable `MCRT_GB300_LIB`.
"""
module MCRTGB300

import MonteCarloRadiativeTransfer as MCRT

const libmcrt = get(ENV, "MCRT_GB300_LIB",
                    joinpath(@__DIR__, "..", "mcrt_gb300", "_lib", "libmcrt.so"))

# ---------------------------------------------------------------- C structs (include/mcrt.h)
struct ScattererDesc            # mcrt_scatterer_desc
    kind::Cint
    omega::Float64
    kl::Float64
    n_theta::Cint
    F11::Ptr{Float64}
    F12::Ptr{Float64}
    F33::Ptr{Float64}
    F34::Ptr{Float64}
    S11::Ptr{Float64}           # ComplexF64 vectors are interleaved (re, im)
    S22::Ptr{Float64}
    random_points::Cint
    csrn::Ptr{Float64}
end

struct ConfigC                  # mcrt_config
    number_of_rays::Int64
    minimum_intensity::Float64
    maximum_scattering_times::Int64
    maximum_threads::Int64
    compute_cb::Cint
    tau0::Float64
    n_phi::Cint
    cos_phi::Ptr{Float64}
    sin_phi::Ptr{Float64}
    n_theta::Cint
    cos_theta::Ptr{Float64}
    sin_theta::Ptr{Float64}
    inorm::Ptr{Float64}
    n_theta_b::Cint
    cos_theta_b::Ptr{Float64}
    sin_theta_b::Ptr{Float64}
    n_phi_b::Cint
    cos_phi_b::Ptr{Float64}
    sin_phi_b::Ptr{Float64}
end

struct LayerC                   # mcrt_layer
    tau::Float64
    omega::Float64
    infinite::Cint
    scatterer::Ptr{Cvoid}
end

struct GeometryC                # mcrt_geometry
    kind::Cint
    theta::Float64
    phi::Float64
    n_layers::Cint
    layers::Ptr{LayerC}
end

struct RunOpts                  # mcrt_run_opts
    precision::Cint             # 0 FP32, 1 FP64
    kernel::Cint                # 0 persistent, 1 plain
    seed::UInt64
    instance::UInt32
    rng_mode::Cint
    photon_begin::Int64
    block_size::Cint
    blocks_per_sm::Cint
    plain_threads::Cint
    table_staging::Cint
    max_attempts::Int64         # 0 = the default rejection-loop cap
end

RunOpts(; precision = 0, kernel = 0, seed = rand(UInt64), instance = 0) =
    RunOpts(precision, kernel, seed, instance, 0, 0, 0, 0, 0, 0, 0)

# ---------------------------------------------------------------- context and errors
const CTX = Ref{Ptr{Cvoid}}(C_NULL)
const SCATTERERS = IdDict{Any, Ptr{Cvoid}}()

function check(rc::Cint)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:mcrt_last_error, libmcrt), Cstring, ()))
    rc == 1 && throw(ArgumentError(msg))     # MCRT_EINVAL: validate() failures
    error("libmcrt error $rc: $msg")
end

function context()
    if CTX[] == C_NULL
        check(ccall((:mcrt_ctx_create, libmcrt), Cint, (Cint, Ref{Ptr{Cvoid}}), 0, CTX))
    end
    return CTX[]
end

function handle(s::MCRT.RayleighScatterer)
    get!(SCATTERERS, s) do
        d = ScattererDesc(0, s.ω, s.kl, 0, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, 0, C_NULL)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:mcrt_scatterer_create, libmcrt), Cint,
                    (Ptr{Cvoid}, Ref{ScattererDesc}, Ref{Ptr{Cvoid}}), context(), d, h))
        h[]
    end
end

function handle(s::MCRT.MieScatterer)
    get!(SCATTERERS, s) do
        F11, F12, F33, F34 = (collect(Float64, v) for v in (s.F11, s.F12, s.F33, s.F34))
        S11, S22 = collect(ComplexF64, s.S11), collect(ComplexF64, s.S22)
        csrn = collect(Float64, s.csrn)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        GC.@preserve F11 F12 F33 F34 S11 S22 csrn begin
            d = ScattererDesc(1, s.ω, s.kl, length(F11), pointer(F11), pointer(F12), pointer(F33),
                              pointer(F34), Ptr{Float64}(pointer(S11)), Ptr{Float64}(pointer(S22)),
                              length(csrn) - 1, pointer(csrn))
            check(ccall((:mcrt_scatterer_create, libmcrt), Cint,
                        (Ptr{Cvoid}, Ref{ScattererDesc}, Ref{Ptr{Cvoid}}), context(), d, h))
        end
        h[]
    end
end

layers_c(g::MCRT.PlaneGeometry) =
    [LayerC(l.τ, l.ω, Cint(isinf(l)), handle(l.scatterer)) for l in g.layers]
layers_c(g::MCRT.SphereGeometry) = [LayerC(g.τ, g.ω, 0, handle(g.scatterer))]
geometry_kind(::MCRT.PlaneGeometry) = 0
geometry_kind(::MCRT.SphereGeometry) = 1
incidence(g::MCRT.PlaneGeometry) = (g.θ, g.ϕ)
incidence(::MCRT.SphereGeometry) = (Float64(π), 0.0)

# Marshals cfg and g into the C structs and calls f(c, gc) while the arrays are alive.
function with_c(f, cfg::MCRT.Config, g)
    arrays = map(a -> collect(Float64, a),
                 (cfg.cosϕ, cfg.sinϕ, cfg.cosθ, cfg.sinθ, cfg.inorm, cfg.cosθb, cfg.sinθb,
                  cfg.cosϕb, cfg.sinϕb))
    Ls = layers_c(g)
    θ, ϕ = incidence(g)
    GC.@preserve arrays Ls begin
        c = ConfigC(cfg.number_of_rays, cfg.minimum_intensity, cfg.maximum_scattering_times,
                    cfg.maximum_threads, Cint(cfg.compute_cb), cfg.τ₀,
                    cfg.Nϕ, pointer(arrays[1]), pointer(arrays[2]),
                    cfg.Nθ, pointer(arrays[3]), pointer(arrays[4]), pointer(arrays[5]),
                    cfg.Nθb, pointer(arrays[6]), pointer(arrays[7]),
                    cfg.Nϕb, pointer(arrays[8]), pointer(arrays[9]))
        gc = GeometryC(geometry_kind(g), θ, ϕ, length(Ls), pointer(Ls))
        return f(c, gc)
    end
end

"""
    simulate(cfg, g, I₀; precision = 0, seed = rand(UInt64), instance = 0)

The GPU branch of `simulate` (src/MonteCarloRadiativeTransfer.jl:36-56): returns
`(Adt, Aabs, Aref, Atrans, Arem, Irt, Icb)` divided by `number_of_rays`, with
`Irt::Array{Float64,3}` of size (4, Nθ, Nϕ) and `Icb` of size (4, Nθb, Nϕb).
"""
function simulate(cfg::MCRT.Config, g, I₀; precision = 0, seed = rand(UInt64), instance = 0)
    I = collect(Float64, I₀)
    A = zeros(5)
    Irt = zeros(4, cfg.Nθ, cfg.Nϕ)
    Icb = zeros(4, cfg.Nθb, cfg.Nϕb)
    opts = RunOpts(; precision, seed, instance)
    with_c(cfg, g) do c, gc
        check(ccall((:mcrt_simulate, libmcrt), Cint,
                    (Ptr{Cvoid}, Ref{ConfigC}, Ref{GeometryC}, Ptr{Float64}, Ref{RunOpts},
                     Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Cvoid}),
                    context(), c, gc, I, opts, A, Irt, Icb, C_NULL, C_NULL))
    end
    return A[1], A[2], A[3], A[4], A[5], Irt, Icb
end

"""
    run_rt(cfg, g; precision = 0, seed = rand(UInt64))

`run_rt(cfg, g; use_gpu = true)` (src/MonteCarloRadiativeTransfer.jl:87-291): the RT and
CB Mueller-matrix DataFrames, with all incident polarisation states in one batched
launch and the matrices assembled on the device (`mcrt_run_rt`).
"""
function run_rt(cfg::MCRT.Config, g; precision = 0, seed = rand(UInt64))
    plane = g isa MCRT.PlaneGeometry
    nrt = cfg.Nθ * (plane ? cfg.Nϕ : 1)
    ncb = cfg.Nθb * (plane ? cfg.Nϕb : 1)
    Mrt = zeros(nrt, 16)            # C layout [16][rows] is Julia's (rows, 16)
    Mcb = zeros(ncb, 16)
    E = zeros(5)
    opts = RunOpts(; precision, seed, instance = 0)
    with_c(cfg, g) do c, gc
        check(ccall((:mcrt_run_rt, libmcrt), Cint,
                    (Ptr{Cvoid}, Ref{ConfigC}, Ref{GeometryC}, Ref{RunOpts}, Ptr{Float64},
                     Ptr{Float64}, Ptr{Float64}, Ptr{Cvoid}),
                    context(), c, gc, opts, Mrt, Mcb, E, C_NULL))
    end
    cols(M) = [Symbol(:s, i, j) => M[:, 4 * (i - 1) + j] for i in 1:4 for j in 1:4]
    θ = 180.0 / π * acos.(collect(cfg.cosθ))
    θb = 180.0 / π * acos.(collect(cfg.cosθb))
    if plane
        SM_rt = MCRT.DataFrame(:θ => repeat(θ; outer = cfg.Nϕ),
                               :ϕ => repeat(180.0 / π * collect(cfg.ϕ); inner = cfg.Nθ), cols(Mrt)...)
        SM_cb = MCRT.DataFrame(:θ => repeat(θb; outer = cfg.Nϕb),
                               :ϕ => repeat(180.0 / π * collect(cfg.ϕb); inner = cfg.Nθb), cols(Mcb)...)
    else
        SM_rt = MCRT.DataFrame(:θ => θ, cols(Mrt)...)
        SM_cb = MCRT.DataFrame(:θ => θb, cols(Mcb)...)
    end
    return SM_rt, SM_cb
end

end # module
