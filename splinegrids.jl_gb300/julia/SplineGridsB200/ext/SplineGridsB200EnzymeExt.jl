"""
Reverse-mode rule for Enzyme (0.13, EnzymeRules) on `evaluate_into!`.

The reference differentiates `evaluate!` by running Enzyme through its KernelAbstractions
kernels (ext/SplineGridsEnzymeExt.jl, test/test_EnzymeExt.jl:14-60).  Enzyme cannot see
into a `ccall`, so the derivative is given here: eval = M * control_points is linear in
the control points, and its adjoint is the library's `sg_evaluate_adjoint`.

    forward:  eval = M * cp                       (the primal, sg_evaluate)
    reverse:  cp_bar += M' * eval_bar ; eval_bar = 0   (eval was overwritten)

The grid is read only (its basis tables and plan), so its shadow gets nothing.  NURBS
grids are not linear in the control points and have no adjoint, as in the reference
(src/adjoint.jl:57); their reverse pass raises.
"""
module SplineGridsB200EnzymeExt

using CUDA
using Enzyme
using Enzyme.EnzymeRules
using SplineGridsB200: evaluate_into!, adjoint_into!

function EnzymeRules.augmented_primal(config::EnzymeRules.RevConfigWidth{1},
        func::Const{typeof(evaluate_into!)}, ::Type{<:Const},
        eval::Annotation{<:CuArray}, grid::Annotation, control_points::Annotation{<:CuArray},
        derivative_order::Const)
    func.val(eval.val, grid.val, control_points.val, derivative_order.val)
    return EnzymeRules.AugmentedReturn(nothing, nothing, nothing)
end

function EnzymeRules.reverse(config::EnzymeRules.RevConfigWidth{1},
        func::Const{typeof(evaluate_into!)}, ::Type{<:Const}, tape,
        eval::Annotation{<:CuArray}, grid::Annotation, control_points::Annotation{<:CuArray},
        derivative_order::Const)
    if !(eval isa Const)
        if !(control_points isa Const)
            # the adjoint overwrites its output: accumulate through a temporary
            tmp = similar(control_points.dval)
            adjoint_into!(tmp, grid.val, eval.dval, derivative_order.val)
            control_points.dval .+= tmp
        end
        fill!(eval.dval, zero(eltype(eval.dval)))
    end
    return (nothing, nothing, nothing, nothing)
end

end # module SplineGridsB200EnzymeExt
