"""splinegrids -- Python host mirror of SplineGrids.jl's API over libsplinegrids_b200.

Names follow the reference (SouthEndMusic/SplineGrids.jl v0.1.1); Julia's mutating
`f!` is spelled `f_`.  Arrays are column-major CUDA tensors with the Julia shape
(see `splinegrids.arrays`); dimension arguments are 0-based, index arrays that the
kernels consume (sample indices, refinement indices) keep the reference's 1-based
values.  All compute runs in the CUDA library; there is no CPU fallback.
"""
from . import arrays, autograd
from ._lib import SplineGridsError, load as load_library
from .batch import GridBatch, GridBatchPipeline
from .fit import FitLoop, batch_fit, grid_fit
from .linear_map import LinearMap, LSQRSolver, lsqr
from .control_points import (DefaultControlPoints, LocalRefinement, LocallyRefinedControlPoints,
                             activate_local_refinement_, deactivate_overwritten_control_points_,
                             evaluate_adjoint_control_points_, evaluate_control_points_,
                             get_n_control_points, local_refinement_, local_refinement_adjoint_,
                             mult_, mult_adjoint_, obtain)
from .refinement import (activate_local_control_point_range_, add_default_local_refinement,
                         error_informed_local_refinement_, insert_knot, insert_knot_grid, refine,
                         refine_dimension, refinement_matrix_device)
from .refinement_matrix import (RefinementMatrix, expand_knots, insert_knot_values,
                                knot_insertion_matrix, knot_span_sequence, refine_knots, rmeye)
from .spline_dimension import (KnotVector, SplineDimension, decompress, evaluate_dimension_,
                               julia_range, set_sample_indices_)
from .spline_grid import (NURBSGrid, SplineGrid, evaluate_, evaluate_adjoint_, evaluate_multi_,
                          set_unit_cp_grid_, tune_adjoint_, validate_partial_derivatives)


def evaluate(obj, *args, **kwargs):
    """Dispatch like the reference's `evaluate!` on the argument type."""
    if isinstance(obj, SplineGrid):
        return evaluate_(obj, *args, **kwargs)
    if isinstance(obj, SplineDimension):
        return evaluate_dimension_(obj)
    return evaluate_control_points_(obj)


def evaluate_adjoint(obj, *args, **kwargs):
    """Dispatch like the reference's `evaluate_adjoint!` on the argument type."""
    if isinstance(obj, SplineGrid):
        return evaluate_adjoint_(obj, *args, **kwargs)
    return evaluate_adjoint_control_points_(obj)


__all__ = [
    "arrays", "autograd", "SplineGridsError", "load_library", "GridBatch", "DefaultControlPoints", "LocalRefinement",
    "LocallyRefinedControlPoints", "activate_local_refinement_",
    "deactivate_overwritten_control_points_", "evaluate_adjoint_control_points_",
    "evaluate_control_points_", "get_n_control_points", "local_refinement_",
    "local_refinement_adjoint_", "mult_", "mult_adjoint_", "obtain",
    "activate_local_control_point_range_", "add_default_local_refinement",
    "error_informed_local_refinement_", "insert_knot", "insert_knot_grid", "refine",
    "refine_dimension", "RefinementMatrix", "expand_knots", "insert_knot_values",
    "knot_insertion_matrix", "refine_knots", "rmeye", "KnotVector",
    "SplineDimension", "decompress", "evaluate_dimension_", "julia_range",
    "set_sample_indices_", "NURBSGrid", "SplineGrid", "evaluate_", "evaluate_adjoint_",
    "set_unit_cp_grid_", "validate_partial_derivatives", "evaluate", "evaluate_adjoint",
    "LinearMap", "LSQRSolver", "lsqr", "evaluate_multi_", "knot_span_sequence",
    "refinement_matrix_device", "GridBatchPipeline", "tune_adjoint_", "FitLoop", "batch_fit",
    "grid_fit",
]
