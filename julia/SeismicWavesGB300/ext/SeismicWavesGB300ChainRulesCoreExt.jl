# A ChainRulesCore rule for the misfit of a simulation: ChainRules-based AD
# systems (Zygote, Diffractor, Enzyme's rule import) differentiate the misfit
# with respect to the material properties through one swgradient! call, which
# gives the misfit and the adjoint gradient together.  SeismicWaves.jl defines
# no AD rules of its own.
#
# Sign: swgradient! returns -dchi/dm on the acoustic simulations (the adjoint
# source is the negated dchi/du, src/models/acoustic/acou_gradient.jl:48,142)
# and +dchi/dm on the elastic one; the pullback returns the derivative itself.
module SeismicWavesGB300ChainRulesCoreExt

using SeismicWaves, ChainRulesCore
using SeismicWaves: WaveSimulation, AcousticWaveSimulation, ElasticWaveSimulation, calcmisfit

gradient_sign(::AcousticWaveSimulation) = -1
gradient_sign(::ElasticWaveSimulation) = 1

tangent_fields(::VpAcousticCDMaterialProperties, g) = (vp = g["vp"],)
tangent_fields(::VpRhoAcousticVDMaterialProperties, g) = (vp = g["vp"], rho = g["rho"])
tangent_fields(::ElasticIsoMaterialProperties, g) = (λ = g["lambda"], μ = g["mu"], ρ = g["rho"])

# wavesim built with gradient = true (any GradParameters)
function ChainRulesCore.rrule(::typeof(swmisfit!), wavesim::WaveSimulation{T, N},
                              matprop::MaterialProperties{T, N}, shots::Vector{<:Shot{T}},
                              misfit::Vector{<:AbstractMisfit{T}}) where {T, N}
    out = swgradient!(wavesim, matprop, shots, misfit)
    g, chi = out isa Tuple ? out : (out, sum(calcmisfit(m, s.recs) for (s, m) in zip(shots, misfit)))
    s = gradient_sign(wavesim)
    function swmisfit_pullback(dchi)
        d = unthunk(dchi)
        fields = map(x -> (s * d) .* x, tangent_fields(matprop, g))
        return NoTangent(), NoTangent(), Tangent{typeof(matprop)}(; fields...), NoTangent(), NoTangent()
    end
    return chi, swmisfit_pullback
end

end # module
