"""Knot insertion, refinement and local-refinement management
(src/refinement.jl, src/control_points.jl:358-578).

These build the structures the hot path consumes (set-up work).  The refinement
matrices are built on the host (small, once); the control-point updates (mult!) and
error-informed refinement (adjoint, reduction, threshold, compaction) run on the device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib, arrays
from .control_points import (DefaultControlPoints, LocalRefinement, LocallyRefinedControlPoints,
                             _workspace, activate_local_refinement_, cartesian_indices,
                             index_tensor, mult_, obtain)
from .refinement_matrix import RefinementMatrix, insert_knot_values, knot_span_sequence
from .spline_dimension import KnotVector, SplineDimension, evaluate_dimension_, set_sample_indices_
from .spline_grid import SplineGrid, evaluate_adjoint_


def insert_knot_vector(knot_vector: KnotVector, knot_new):
    """insert_knot(knot_vector, knot_new) (src/refinement.jl:90-133): the new knot vector
    and the 1-based knot span index of the inserted knot."""
    kv, mult, ksi = insert_knot_values(knot_vector.knot_values.cpu().numpy(),
                                       knot_vector.multiplicities.cpu().numpy(), knot_new)
    return KnotVector(torch.as_tensor(kv), torch.as_tensor(mult),
                      device=knot_vector.knots_all.device), ksi


def _dimension_like(dim: SplineDimension, knot_vector: KnotVector, *, recompute: bool,
                    evaluate: bool) -> SplineDimension:
    """setproperties(spline_dimension; knot_vector) with fresh index/basis arrays."""
    new = SplineDimension.__new__(SplineDimension)
    new.degree = dim.degree
    new.max_derivative_order = dim.max_derivative_order
    new.knot_vector = knot_vector
    new.sample_points = dim.sample_points
    new.sample_indices = dim.sample_indices.clone()
    new.eval = arrays.zeros(tuple(dim.eval.shape), dim.eval.dtype, dim.eval.device)
    if recompute:
        set_sample_indices_(new)
        if evaluate:
            evaluate_dimension_(new)
    return new


def refinement_matrix_device(knots_all: torch.Tensor, degree: int, knots_new,
                             knot_span_indices) -> RefinementMatrix:
    """The refinement matrix of inserting ``knots_new`` in order (``knot_span_indices``:
    1-based span of each knot in the knot vector at its insertion), built on the device
    in one launch (sg_refine_matrix): the composition R_k ... R_1 of the single-knot
    matrices of src/refinement.jl:3-36 with the banded product of
    src/refinement_matrix.jl:184-327, bit-identical to composing them one by one.  The
    device arrays stay cached on the returned matrix for mult!."""
    dev, dt = knots_all.device, knots_all.dtype
    nk = knots_all.numel()
    n_ins = len(knots_new)
    rows = nk - degree - 1 + n_ins
    kn = torch.as_tensor(np.asarray(knots_new), dtype=dt).to(dev).contiguous()
    ks = torch.as_tensor(np.asarray(knot_span_indices, dtype=np.int32)).to(dev).contiguous()
    rp = torch.empty(max(rows, 1), dtype=torch.int32, device=dev)
    cs = torch.empty(max(rows, 1), dtype=torch.int32, device=dev)
    nz = torch.empty(max(rows * (degree + 2), 1), dtype=dt, device=dev)
    code = arrays.dtype_code(dt)
    lib = _lib.load()
    ws = torch.empty(int(lib.sg_refine_matrix_workspace_bytes(code, degree, nk, n_ins)),
                     dtype=torch.uint8, device=dev)
    nnz = C.c_int64(0)
    _lib.check(lib.sg_refine_matrix(code, int(degree), knots_all.contiguous().data_ptr(), nk, n_ins,
                                    kn.data_ptr() if n_ins else None,
                                    ks.data_ptr() if n_ins else None, rp.data_ptr(), cs.data_ptr(),
                                    nz.data_ptr(), C.byref(nnz), ws.data_ptr(),
                                    _lib.stream_handle()))
    k = int(nnz.value)
    rm = RefinementMatrix(rows, nk - degree - 1, rp[:rows].cpu().numpy(), cs[:rows].cpu().numpy(),
                          nz[:k].cpu().numpy(), validate=False)
    rm._dev[(str(dev), dt)] = (rp[:rows], cs[:rows], nz[:k])
    return rm


def insert_knot(spline_dimension: SplineDimension, knot_new, *,
                recompute_sample_indices: bool = True, evaluate: bool = True):
    """insert_knot(::SplineDimension, knot_new) (src/refinement.jl:135-186); the matrix is
    built on the device."""
    kv_new, ksi = insert_knot_vector(spline_dimension.knot_vector, knot_new)
    kn = spline_dimension.knot_vector.knots_all
    rm = refinement_matrix_device(kn, spline_dimension.degree,
                                  [kn.new_tensor(float(knot_new)).item()], [ksi])
    new = _dimension_like(spline_dimension, kv_new, recompute=recompute_sample_indices,
                          evaluate=evaluate)
    return new, rm


def refine_dimension(spline_dimension: SplineDimension, knots_new=None):
    """refine(::SplineDimension; knots_new) (src/refinement.jl:237-284): insert every knot
    (default: the midpoints of the knot spans) and compose the refinement matrices.
    The knot values and spans are bookkept on the host (a few numbers per knot); the
    matrix is built on the device in one launch (refinement_matrix_device); the new
    dimension's sample indices are recomputed on the device, its basis table is
    evaluated by the caller."""
    kv0 = spline_dimension.knot_vector
    kv, mult, knots, spans = knot_span_sequence(kv0.knot_values.cpu().numpy(),
                                                kv0.multiplicities.cpu().numpy(), knots_new)
    rm = refinement_matrix_device(kv0.knots_all, spline_dimension.degree, knots, spans)
    kv_new = KnotVector(torch.as_tensor(kv), torch.as_tensor(mult), device=kv0.knots_all.device)
    new = _dimension_like(spline_dimension, kv_new, recompute=True, evaluate=False)
    return new, rm


def _refine_grid(grid: SplineGrid, dim_new: SplineDimension, dim: int, rm: RefinementMatrix):
    """refine(grid, spline_dimension_new, dim_refinement, refinement_matrix)
    (src/refinement.jl:332-386): new grid whose control points are mult!(R, cps)."""
    assert not grid.is_nurbs(), "Knot insertion not supported for NURBS"
    cp = obtain(grid.control_points)
    size_new = list(cp.shape)
    size_new[dim] += rm.m - rm.n
    cp_new = arrays.empty(size_new, cp.dtype, cp.device)
    mult_(cp_new, (rm,), cp, (dim,))
    dims = tuple(dim_new if k == dim else d for k, d in enumerate(grid.spline_dimensions))
    return SplineGrid(dims, control_points=DefaultControlPoints(cp_new)), rm


def insert_knot_grid(grid: SplineGrid, dim_refinement: int, knot_new, *,
                     evaluate_spline_dimension: bool = True):
    """insert_knot(spline_grid, dim_refinement, knot_new) (src/refinement.jl:188-235);
    dim_refinement is 0-based."""
    assert not grid.is_nurbs(), "Knot insertion not supported for NURBS"
    d_new, rm = insert_knot(grid.spline_dimensions[dim_refinement], knot_new,
                            evaluate=evaluate_spline_dimension)
    return _refine_grid(grid, d_new, dim_refinement, rm)


def refine(grid: SplineGrid, dim_refinement: int, knots_new=None):
    """refine(spline_grid, dim_refinement; knots_new) (src/refinement.jl:286-330);
    dim_refinement is 0-based."""
    assert not grid.is_nurbs(), "Knot insertion not supported for NURBS"
    d_new, rm = refine_dimension(grid.spline_dimensions[dim_refinement], knots_new)
    evaluate_dimension_(d_new)
    return _refine_grid(grid, d_new, dim_refinement, rm)


def add_default_local_refinement(grid: SplineGrid) -> SplineGrid:
    """add_default_local_refinement (src/control_points.jl:358-425): bisect every knot span
    in every dimension and add a level of LocallyRefinedControlPoints (no control points
    activated yet)."""
    cps = grid.control_points
    cp = obtain(cps)
    dims_new, mats = [], []
    for d in grid.spline_dimensions:
        dn, rm = refine_dimension(d)
        dims_new.append(dn)
        mats.append(rm)
    for dn in dims_new:
        evaluate_dimension_(dn)
    nin, nout = grid.nin, grid.nout
    size_new = tuple(dn.n_basis_functions for dn in dims_new) + (nout,)
    cp_new = arrays.zeros(size_new, cp.dtype, cp.device)
    mult_(cp_new, tuple(mats), cp, tuple(range(nin)))
    lr = LocalRefinement(list(range(nin)), mats,
                         arrays.empty((0, nin), torch.int32, cp.device),
                         arrays.empty((0, nout), cp.dtype, cp.device))
    if isinstance(cps, DefaultControlPoints):
        ncp = cps.n_control_points()
        base_idx = index_tensor(cartesian_indices(cp.shape[:-1]), cp.device)
        base_vals = arrays.empty((ncp, nout), cp.dtype, cp.device)
        base_vals.copy_(cps.values_matrix())
        base = LocalRefinement([], [], base_idx, base_vals)
        new_cps = LocallyRefinedControlPoints([cp, cp_new], [base, lr])
    else:
        cps.control_points_refined.append(cp_new)
        cps.local_refinements.append(lr)
        new_cps = cps
    return SplineGrid(tuple(dims_new), control_points=new_cps, weights=grid.weights)


def activate_local_control_point_range_(grid: SplineGrid, *ranges) -> None:
    """activate_local_control_point_range! (src/control_points.jl:527-539): activate the
    product of per-dimension 0-based Python ranges (first range fastest)."""
    assert len(ranges) == grid.nin
    grids = np.meshgrid(*[np.asarray(list(r)) + 1 for r in ranges], indexing="ij")
    idx = np.stack([g.flatten(order="F") for g in grids], axis=1).astype(np.int32)
    activate_local_refinement_(grid.control_points, idx)


def error_informed_local_refinement_(grid: SplineGrid, error: torch.Tensor,
                                     threshold_factor: float = 1.0) -> None:
    """error_informed_local_refinement! (src/control_points.jl:541-578) on the device: map
    the error onto the finest control points with the adjoint, sum over outputs, and
    activate (at the last level) every control point above threshold_factor * mean that
    the level does not overwrite yet, in findall order, with its current value."""
    assert tuple(error.shape) == tuple(grid.eval.shape), \
        "The error array must have the same size as the eval array."
    cps = grid.control_points
    if not isinstance(cps, LocallyRefinedControlPoints):
        raise TypeError("error_informed_local_refinement! needs locally refined control points "
                        "(add_default_local_refinement)")
    dev, dt = error.device, grid.dtype
    finest = obtain(cps)
    cp_err = arrays.zeros(tuple(finest.shape), dt, dev)
    evaluate_adjoint_(grid, eval=error, control_points=cp_err)
    shape = tuple(finest.shape[:-1])
    nin, nout = len(shape), finest.shape[-1]
    ncp = int(np.prod(shape))
    lib = _lib.load()
    ws = _workspace(ncp, dev)
    per_cp = torch.empty(max(ncp, 1), dtype=dt, device=dev)
    total = torch.zeros(1, dtype=torch.float64, device=dev)
    stream = _lib.stream_handle()
    _lib.check(lib.sg_sum_outputs(arrays.dtype_code(dt), ncp, nout, arrays.ptr(cp_err, "error"),
                                  per_cp.data_ptr(), total.data_ptr(), ws.data_ptr(), stream))
    lrs = cps.local_refinements
    level = len(lrs) - 1
    lr = lrs[level]
    out_idx = arrays.empty((max(ncp, 1), nin), torch.int32, dev)
    out_vals = arrays.empty((max(ncp, 1), nout), dt, dev)
    n_sel = C.c_int64(0)
    old = lr.refinement_indices
    _lib.check(lib.sg_select_above(
        arrays.dtype_code(dt), nin, _lib.i64_array(shape), nout, per_cp.data_ptr(),
        total.data_ptr(), float(threshold_factor),
        arrays.ptr(old, "refinement_indices") if lr.n_refined else None, lr.n_refined,
        arrays.ptr(finest, "control_points"), arrays.ptr(out_idx, "indices"),
        arrays.ptr(out_vals, "values"), C.byref(n_sel), ws.data_ptr(), stream))
    k = int(n_sel.value)
    n_old = lr.n_refined
    idx = arrays.empty((n_old + k, nin), torch.int32, dev)
    vals = arrays.empty((n_old + k, nout), dt, dev)
    if n_old:
        idx[:n_old].copy_(old)
        vals[:n_old].copy_(lr.refinement_values)
    if k:
        idx[n_old:].copy_(out_idx[:k])
        vals[n_old:].copy_(out_vals[:k])
    lrs[level] = LocalRefinement(lr.dims_refinement, lr.refinement_matrices, idx, vals)
