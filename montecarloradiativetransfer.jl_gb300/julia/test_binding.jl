# Parity of the libmcrt binding (MCRTGB300.jl) against the package's own CPU path:
# MonteCarloRadiativeTransfer.simulate(cfg, g, I₀; use_gpu = false) against
# MCRTGB300.simulate(cfg, g, I₀) on the same configurations. For a maintainer with
# Julia (>= 1.9), the package and a GB300:
#
#     julia --project=<MonteCarloRadiativeTransfer.jl checkout> test_binding.jl
#
# with MCRT_GB300_LIB set to libmcrt.so unless this folder sits in the built tree.
#
# The two paths draw different random numbers, so the check is statistical, by batch
# means over independent runs: the energy fractions, the intensity summed over azimuths
# in every polar bin and the CB peak (s11 of Icb at θb = 0) agree within 5 combined
# standard errors; quantities with no spread (direct transmission of a slab) agree to
# rounding. It also checks that an invalid geometry raises the package's ArgumentError.

using Test
import MonteCarloRadiativeTransfer as MCRT

include(joinpath(@__DIR__, "MCRTGB300.jl"))

const NB = 8  # independent runs per path

function observables(res)
    Adt, Aabs, Aref, Atrans, Arem, Irt, Icb = res
    return vcat([Adt, Aabs, Aref, Atrans, Arem], vec(sum(Irt[1, :, :]; dims = 2)), [Icb[1, 1, 1]])
end

# mean and standard error over the runs, per observable
function batch_means(rows)
    X = reduce(hcat, rows)
    n = size(X, 2)
    μ = vec(sum(X; dims = 2)) ./ n
    σ = sqrt.(vec(sum((X .- μ) .^ 2; dims = 2)) ./ (n - 1) ./ n)
    return μ, σ
end

function compare(name, cfg, g; I₀ = [1.0, 0.0, 0.0, 0.0])
    μc, σc = batch_means([observables(MCRT.simulate(cfg, g, I₀; use_gpu = false)) for _ in 1:NB])
    μg, σg = batch_means([observables(MCRTGB300.simulate(cfg, g, I₀; precision = 1)) for _ in 1:NB])
    spread = sqrt.(σc .^ 2 .+ σg .^ 2)
    live = spread .> 0
    z = (μc[live] .- μg[live]) ./ spread[live]
    @info name max_abs_z = maximum(abs, z)
    @test all(abs.(z) .< 5)
    @test all(isapprox.(μc[.!live], μg[.!live]; rtol = 1e-10, atol = 1e-14))
end

@testset "MCRTGB300 against the package's CPU path" begin
    ray = MCRT.RayleighScatterer(0.9, 1.0)
    plane = MCRT.PlaneGeometry(5π / 6, 0.0, [MCRT.Layer(d = 1.0, scatterer = ray)])
    compare("Rayleigh slab", MCRT.Config(geometry = plane, number_of_rays = 2000, Nθ = 16, Nϕ = 8), plane)

    mie = MCRT.MieScatterer(2 / 2π, 1.5 + 0.01im, 1.0, 0.1; Nθ = 1801)
    slab = MCRT.PlaneGeometry(5π / 6, 0.0, [MCRT.Layer(d = mie.kl, scatterer = mie)])
    compare("Mie slab", MCRT.Config(geometry = slab, number_of_rays = 2000, Nθ = 16, Nϕ = 8), slab)

    sphere = MCRT.SphereGeometry(R = 2.0, scatterer = ray)
    compare("Rayleigh sphere", MCRT.Config(geometry = sphere, number_of_rays = 2000, Nθ = 16, Nϕ = 8), sphere)

    bad = MCRT.PlaneGeometry(1.0, 0.0, plane.layers)  # θ outside (π/2, π]
    @test_throws ArgumentError MCRTGB300.simulate(MCRT.Config(geometry = bad), bad, [1.0, 0.0, 0.0, 0.0])
end
