"""
The reference's `solve(prob, Tsit5(); saveat, ...)` and `solve(prob, TRBDF2(...))` (src/solve.jl:197-220;
src/specific_problems/abstract_templates.jl:58-60) on the GPU: methods of `CommonSolve.solve`
for an `FVMProblem`, an `FVMSystem` and the time-dependent templates with OrdinaryDiffEq's
`Tsit5`, more specific than the reference's own, so an unchanged script that loads
FiniteVolumeMethodGPU runs its Tsit5 solves through libfvmgpu.  The result is a SciMLBase
`ODESolution` of the saved states (`sol.t`, `sol.u`, `sol[k]`).  Without `saveat` the initial
and final states are saved (the reference would save every step).  Keywords: `saveat`, `dt`
(with `adaptive = false` for fixed steps), `abstol`, `reltol`, `maxiters`; others are ignored.
"""
module FiniteVolumeMethodGPUOrdinaryDiffEqExt

using FiniteVolumeMethodGPU
using FiniteVolumeMethod
using OrdinaryDiffEq: Tsit5, TRBDF2
import CommonSolve
import SciMLBase

const G = FiniteVolumeMethodGPU
const FVM = FiniteVolumeMethod

function gpu_solution(alg, ts, us)
    ode = SciMLBase.ODEProblem((du, u, p, t) -> nothing, copy(us[1]), (first(ts), last(ts)))
    return SciMLBase.build_solution(ode, alg, ts, us; retcode = SciMLBase.ReturnCode.Success)
end

save_times(prob, saveat) = saveat === nothing || (saveat isa AbstractVector && isempty(saveat)) ?
                           [prob.initial_time, prob.final_time] : saveat

function gpu_tsit5(prob, alg; saveat = nothing, dt = nothing, adaptive = true, abstol = 1e-6, reltol = 1e-3,
                   maxiters = 0, kwargs...)
    g = G.gpu_object(prob)
    fixed = dt !== nothing && !adaptive
    ts, us = G.solve(g; saveat = save_times(prob, saveat), dt = fixed ? dt : nothing, abstol, reltol,
                     max_steps = maxiters)
    return gpu_solution(alg, ts, us)
end

CommonSolve.solve(prob::FVM.FVMProblem, alg::Tsit5; kwargs...) = gpu_tsit5(prob, alg; kwargs...)

# TRBDF2 (the tutorials' implicit method, whatever linsolve it names): the device's TR-BDF2
function gpu_trbdf2(prob, alg; saveat = nothing, dt = nothing, adaptive = true, abstol = 1e-6, reltol = 1e-3,
                    maxiters = 0, kwargs...)
    g = G.gpu_object(prob)
    fixed = dt !== nothing && !adaptive
    ts, us, _ = G.solve_trbdf2(g; saveat = save_times(prob, saveat), dt = fixed ? dt : nothing, abstol, reltol,
                               max_steps = maxiters)
    return gpu_solution(alg, ts, us)
end
CommonSolve.solve(prob::FVM.FVMProblem, alg::TRBDF2; kwargs...) = gpu_trbdf2(prob, alg; kwargs...)
CommonSolve.solve(sys::FVM.FVMSystem, alg::TRBDF2; kwargs...) = gpu_trbdf2(sys, alg; kwargs...)
CommonSolve.solve(tmpl::FVM.DiffusionEquation, alg::TRBDF2; kwargs...) = gpu_trbdf2(tmpl, alg; kwargs...)
CommonSolve.solve(tmpl::FVM.LinearReactionDiffusionEquation, alg::TRBDF2; kwargs...) = gpu_trbdf2(tmpl, alg; kwargs...)
CommonSolve.solve(sys::FVM.FVMSystem, alg::Tsit5; kwargs...) = gpu_tsit5(sys, alg; kwargs...)
CommonSolve.solve(tmpl::FVM.DiffusionEquation, alg::Tsit5; kwargs...) = gpu_tsit5(tmpl, alg; kwargs...)
CommonSolve.solve(tmpl::FVM.LinearReactionDiffusionEquation, alg::Tsit5; kwargs...) = gpu_tsit5(tmpl, alg; kwargs...)

end # module
