# ChainRulesCore.rrule for GLAGPU.eigen on real symmetric matrices, backed by
# the device adjoint (gla_plan_adjoint_host). Include after GLAGPU.jl in an
# environment that has ChainRulesCore:
#
#     include("GLAGPU.jl"); include("GLAGPUChainRules.jl")
#     Zygote.gradient(A -> sum(abs2, GLAGPU.eigen(Symmetric(A)).vectors[:, 1]), A)
#
# The pullback returns the symmetric cotangent projected onto the input's
# type (ProjectTo), so Symmetric/Hermitian wrappers receive Symmetric/
# Hermitian tangents.
using ChainRulesCore
using LinearAlgebra

function ChainRulesCore.rrule(::typeof(GLAGPU.eigen),
                              A::Union{Hermitian{Float64,Matrix{Float64}},Symmetric{Float64,Matrix{Float64}}})
    E = GLAGPU.eigen(A)
    project = ProjectTo(A)
    function eigen_pullback(dE)
        dE = unthunk(dE)
        wbar = dE.values isa AbstractZero ? nothing : dE.values
        Vbar = dE.vectors isa AbstractZero ? nothing : dE.vectors
        wbar === nothing && Vbar === nothing && return NoTangent(), ZeroTangent()
        return NoTangent(), project(GLAGPU.eigen_adjoint(E, wbar, Vbar))
    end
    return E, eigen_pullback
end
