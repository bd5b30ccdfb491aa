"""
ChainRulesCore `rrule` for the out-of-place `evaluate_cp(grid, control_points)`: the
pullback of eval = M * cp is cp_bar = M' * eval_bar, the library's `sg_evaluate_adjoint`
(deterministic gather form).  For Zygote and the other ChainRules-based AD systems; the
reference's own AD path is Enzyme (ext/SplineGridsEnzymeExt.jl).
"""
module SplineGridsB200ChainRulesCoreExt

using CUDA
using ChainRulesCore
using SplineGridsB200: evaluate_cp, adjoint_into!

function ChainRulesCore.rrule(::typeof(evaluate_cp), grid, control_points::CuArray;
        derivative_order = ntuple(_ -> 0, ndims(control_points) - 1))
    eval = evaluate_cp(grid, control_points; derivative_order)
    function evaluate_cp_pullback(eval_bar)
        eb = unthunk(eval_bar)
        eb isa AbstractZero && return (NoTangent(), NoTangent(), ZeroTangent())
        cp_bar = similar(control_points)
        adjoint_into!(cp_bar, grid, eb isa CuArray ? eb : CuArray(eb), derivative_order)
        return (NoTangent(), NoTangent(), cp_bar)
    end
    return eval, evaluate_cp_pullback
end

end # module SplineGridsB200ChainRulesCoreExt
