"""Reverse-mode differentiation of `evaluate!` with respect to the control points.

The reference differentiates a loss through `evaluate!(spline_grid; control_points)`
with Enzyme (ext/SplineGridsEnzymeExt.jl, test/test_EnzymeExt.jl:14-60), which
differentiates its KernelAbstractions kernels.  Here the derivative of the forward is
the library's adjoint itself (`evaluate_adjoint!`, deterministic gather form), wired
into torch autograd: ``evaluate(grid, control_points)`` returns eval as a tensor whose
backward applies ``evaluate_adjoint_`` to the incoming cotangent.  NURBS grids are not
linear in the control points and have no adjoint (as in the reference), so they are
rejected.
"""
from __future__ import annotations

import torch

from . import arrays
from .control_points import obtain
from .spline_grid import SplineGrid, evaluate_, evaluate_adjoint_


class _Evaluate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, control_points, grid, order):
        ev = arrays.empty(tuple(grid.eval.shape), grid.dtype, control_points.device)
        cp = control_points
        if not arrays.is_colmajor(cp):
            cp = arrays.empty(tuple(cp.shape), cp.dtype, cp.device)
            cp.copy_(control_points)
        evaluate_(grid, derivative_order=order, control_points=cp, eval=ev)
        ctx.grid, ctx.order = grid, order
        ctx.cp_shape = tuple(control_points.shape)
        return ev

    @staticmethod
    def backward(ctx, grad_eval):
        grid = ctx.grid
        g = arrays.empty(tuple(grad_eval.shape), grid.dtype, grad_eval.device)
        g.copy_(grad_eval)  # the cotangent in the library's (column-major) layout
        cp_bar = arrays.empty(ctx.cp_shape, grid.dtype, grad_eval.device)
        evaluate_adjoint_(grid, derivative_order=ctx.order, control_points=cp_bar, eval=g)
        return cp_bar, None, None


def evaluate(grid: SplineGrid, control_points: torch.Tensor | None = None,
             derivative_order=None) -> torch.Tensor:
    """eval = evaluate!(grid; derivative_order, control_points) as a differentiable
    function of ``control_points`` (default: the grid's own); returns a new eval tensor."""
    if grid.is_nurbs():
        raise ValueError("Adjoint evaluation not supported for NURBS.")
    cp = obtain(grid.control_points) if control_points is None else control_points
    order = tuple(derivative_order) if derivative_order is not None else (0,) * grid.nin
    return _Evaluate.apply(cp, grid, order)
