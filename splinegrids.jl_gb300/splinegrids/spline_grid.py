"""SplineGrid / NURBSGrid and the grid-level evaluate! / evaluate_adjoint!
(src/spline_grid.jl, src/adjoint.jl:52-83, src/validation.jl).

Every evaluation goes through a cached plan of the library (one per grid and control
point storage type); the plan holds the device scratch of the separable passes, so
evaluate_ and evaluate_adjoint_ allocate nothing.
"""
from __future__ import annotations

import ctypes as C
import logging
import weakref

import numpy as np
import torch

from . import _lib, arrays
from .control_points import DefaultControlPoints, obtain
from .spline_dimension import SplineDimension

log = logging.getLogger("splinegrids")


def set_unit_cp_grid_(control_points: torch.Tensor) -> None:
    """Default control points (src/utils.jl:1-15): output n < min(Nin, Nout) is the
    n-th input coordinate on range(0, 1) over the control-point grid."""
    nin = control_points.dim() - 1
    nout = control_points.shape[-1]
    shp = tuple(control_points.shape[:-1])
    for n in range(min(nin, nout)):
        coords = torch.as_tensor(np.arange(shp[n], dtype=np.float64) / max(shp[n] - 1, 1)
                                 if shp[n] > 1 else np.zeros(1))
        view = [1] * nin
        view[n] = shp[n]
        control_points[..., n].copy_(coords.reshape(view).expand(shp))


class _Plan:
    """Owner of one sg_grid_plan handle."""

    def __init__(self, grid: "SplineGrid", dtype_code: int):
        dims = grid.spline_dimensions
        desc = _lib.GridDesc()
        desc.nin = len(dims)
        desc.nout = grid.nout
        desc.dtype = dtype_code
        desc.has_weights = 1 if grid.weights is not None else 0
        for k, d in enumerate(dims):
            desc.n_samples[k] = len(d)
            desc.n_basis[k] = d.n_basis_functions
            desc.degree[k] = d.degree
            desc.max_derivative_order[k] = d.max_derivative_order
            desc.sample_indices[k] = d.sample_indices.data_ptr()
            desc.basis_eval[k] = arrays.ptr(d.eval, "basis table")
        self.desc = desc
        h = C.c_void_p()
        _lib.check(_lib.load().sg_grid_plan_create(C.byref(desc), _lib.stream_handle(),
                                                   C.byref(h)))
        self.handle = h
        self._fin = weakref.finalize(self, _lib.load().sg_grid_plan_destroy, h)

    def workspace_bytes(self) -> int:
        return int(_lib.load().sg_grid_plan_workspace_bytes(self.handle))

    def enable_timing(self, on: bool = True) -> None:
        """Record CUDA events around every kernel launch of later calls."""
        _lib.check(_lib.load().sg_grid_plan_enable_timing(self.handle, 1 if on else 0))

    def pass_times(self) -> list:
        """Durations (ms) of the passes of the last timed call, in launch order."""
        cap = C.c_int32(_lib.SG_MAX_NIN)
        ms = (C.c_float * _lib.SG_MAX_NIN)()
        _lib.check(_lib.load().sg_grid_plan_pass_times(self.handle, ms, C.byref(cap)))
        return [float(ms[i]) for i in range(cap.value)]

    def check(self) -> None:
        """Synchronize and raise if a bounded device wait of an earlier call gave up."""
        _lib.check(_lib.load().sg_grid_plan_check(self.handle, _lib.stream_handle()))

    def tune(self, derivative_order, eval_bar: torch.Tensor, control_points_bar: torch.Tensor):
        """Time the adjoint stream's chunk-size candidates on these arrays (scratch) and
        keep the fastest per axis; returns the choice per axis (0: heuristic)."""
        chosen = (C.c_int32 * _lib.SG_MAX_NIN)()
        _lib.check(_lib.load().sg_grid_plan_tune(
            self.handle, _lib.i32_array(derivative_order), arrays.ptr(eval_bar, "eval"),
            arrays.ptr(control_points_bar, "control_points"), _lib.stream_handle(), chosen))
        return [int(chosen[k]) for k in range(len(derivative_order))]

    def untune(self) -> None:
        _lib.check(_lib.load().sg_grid_plan_untune(self.handle))

    STRATEGIES = {"auto": 0, "separable": 1, "fused": 2}

    def set_strategy(self, strategy: str) -> None:
        """"auto" (fused wherever it applies), "separable" (one launch per axis) or
        "fused" (Nin = 2: both axes in one launch); results are bitwise the same."""
        _lib.check(_lib.load().sg_grid_plan_set_strategy(self.handle, self.STRATEGIES[strategy]))

    def paths(self) -> tuple:
        """The path ("separable" / "fused") of evaluate and of evaluate_adjoint."""
        f, a = C.c_int32(), C.c_int32()
        _lib.check(_lib.load().sg_grid_plan_paths(self.handle, C.byref(f), C.byref(a)))
        names = {1: "separable", 2: "fused"}
        return names[f.value], names[a.value]


class SplineGrid:
    """The central object (src/spline_grid.jl:1-117): spline dimensions, control points,
    optional NURBS weights and the eval array [n_samples..., Nout].

    ``SplineGrid(spline_dimensions, Nout)`` builds default (unit grid) control points and
    a zero eval, as the reference.  ``SplineGrid.from_parts(dims, control_points, weights,
    eval)`` is the reference's inner constructor with its validation."""

    def __init__(self, spline_dimensions, nout: int | None = None, *, control_points=None,
                 weights=None, eval=None):
        if isinstance(spline_dimensions, SplineDimension):
            spline_dimensions = (spline_dimensions,)
        self.spline_dimensions = tuple(spline_dimensions)
        d0 = self.spline_dimensions[0]
        dev, tv = d0.eval.device, d0.dtype
        if control_points is None:
            assert nout is not None
            cp = arrays.zeros(self.control_point_grid_size() + (nout,), tv, dev)
            set_unit_cp_grid_(cp)
            control_points = DefaultControlPoints(cp)
        elif isinstance(control_points, torch.Tensor):
            control_points = DefaultControlPoints(control_points)
        if eval is None:
            eval = arrays.zeros(self.sample_grid_size() + (control_points.shape[-1],), tv, dev)
        validate_spline_grid(self.spline_dimensions, control_points, weights, eval)
        self.control_points = control_points
        self.weights = weights
        self.eval = eval
        self._plans = {}

    @classmethod
    def from_parts(cls, spline_dimensions, control_points, weights, eval):
        return cls(spline_dimensions, control_points=control_points, weights=weights, eval=eval)

    # ---------------------------------------------------------------- sizes
    @property
    def nin(self) -> int:
        return len(self.spline_dimensions)

    @property
    def nout(self) -> int:
        return self.control_points.shape[-1]

    @property
    def dtype(self):
        return self.spline_dimensions[0].dtype

    def is_nurbs(self) -> bool:
        return self.weights is not None

    def sample_grid_size(self):
        return tuple(len(d) for d in self.spline_dimensions)

    def control_point_grid_size(self):
        return tuple(d.n_basis_functions for d in self.spline_dimensions)

    def cp_kernel_size(self):
        return tuple(d.degree + 1 for d in self.spline_dimensions)

    def n_control_points(self) -> int:
        return self.control_points.n_control_points()

    # ---------------------------------------------------------------- plans
    def plan(self, cp_dtype: torch.dtype | None = None) -> _Plan:
        tv = self.dtype
        code = arrays.dtype_code(tv)
        if cp_dtype == torch.bfloat16:
            if tv != torch.float32:
                raise TypeError("bfloat16 control points need a Float32 grid")
            code = _lib.SG_BF16_F32
        if code not in self._plans:
            self._plans[code] = _Plan(self, code)
        return self._plans[code]

    def refresh_plans(self) -> None:
        """Re-read sample indices after set_sample_indices_ changed them."""
        for p in self._plans.values():
            _lib.check(_lib.load().sg_grid_plan_refresh(p.handle, _lib.stream_handle()))

    def __repr__(self):
        kind = "NURBSGrid" if self.is_nurbs() else "SplineGrid"
        shape = {1: "curve", 2: "surface", 3: "volume"}.get(self.nin, f"hyper ({self.nin}) volume")
        return f"{kind} {shape} with outputs in R^{self.nout} ({self.dtype})"


def NURBSGrid(spline_dimensions, nout: int) -> SplineGrid:
    """A SplineGrid with weights (ones) on the control-point grid (src/spline_grid.jl:96-108)."""
    g = SplineGrid(spline_dimensions, nout)
    g.weights = arrays.ones(g.control_point_grid_size(), g.dtype, g.eval.device)
    return g


def validate_spline_grid(spline_dimensions, control_points, weights, eval) -> None:
    """validate_spline_grid (src/validation.jl:1-50), with the reference's messages."""
    errors = False
    nin_sd = len(spline_dimensions)
    nin_cp = len(control_points.shape) - 1
    nin_ev = eval.dim() - 1
    if weights is None:
        nins = (nin_sd, nin_cp, nin_ev)
        if len(set(nins)) != 1:
            log.error("The number of input dimensions from the spline dimensions, control_points, "
                      "and eval must agree, got %s respectively.", nins)
            errors = True
    else:
        nins = (nin_sd, nin_cp, nin_ev, weights.dim())
        if len(set(nins)) != 1:
            log.error("The number of input dimensions from the spline dimensions, control_points, "
                      "eval and weights must agree, got %s respectively.", nins)
            errors = True
    if control_points.shape[-1] != eval.shape[-1]:
        log.error("The number of output dimensions from the control points %d and eval %d must "
                  "agree.", control_points.shape[-1], eval.shape[-1])
        errors = True
    cp_sd = tuple(d.n_basis_functions for d in spline_dimensions)
    cp_cp = tuple(control_points.shape[:-1])
    if cp_sd != cp_cp:
        log.error("The control point grid sizes from the spline dimensions %s and the control "
                  "points %s must agree.", cp_sd, cp_cp)
        errors = True
    if errors:
        raise ValueError("Errors encountered when validating spline grid constructor inputs.")


def validate_partial_derivatives(grid_or_dims, derivative_order) -> None:
    """validate_partial_derivatives (src/validation.jl:52-88)."""
    if isinstance(grid_or_dims, SplineGrid):
        if grid_or_dims.is_nurbs():
            if any(o != 0 for o in derivative_order):
                raise ValueError("Computing derivatives of NURBS is currently not supported.")
            return
        dims = grid_or_dims.spline_dimensions
    else:
        dims = grid_or_dims
    errors = False
    for i, (d, o) in enumerate(zip(dims, derivative_order)):
        if not (0 <= o <= d.max_derivative_order):
            errors = True
            log.error("The maximum derivative order available for spline dimension %d is %d, "
                      "got %d.", i + 1, d.max_derivative_order, o)
    if errors:
        raise ValueError("Invalid derivative order(s) supplied. If you want to evaluate (higher "
                         "order) derivatives, specify this at construction as "
                         "SplineDimension(...; max_derivative_order).")


def evaluate_(grid: SplineGrid, derivative_order=None, control_points=None, eval=None) -> None:
    """evaluate!(spline_grid; derivative_order, control_points, eval)
    (src/spline_grid.jl:185-230): eval = sum over the support of the basis product times
    the control points, divided by the weighted denominator for NURBS."""
    order = tuple(derivative_order) if derivative_order is not None else (0,) * grid.nin
    validate_partial_derivatives(grid, order)
    cp = obtain(grid.control_points if control_points is None else control_points)
    ev = grid.eval if eval is None else eval
    assert tuple(cp.shape) == tuple(obtain(grid.control_points).shape)
    assert tuple(ev.shape) == tuple(grid.eval.shape)
    if cp.dtype not in (grid.dtype, torch.bfloat16) or ev.dtype != grid.dtype:
        raise TypeError(f"control points {cp.dtype} / eval {ev.dtype} do not match the grid's "
                        f"{grid.dtype}")
    plan = grid.plan(cp.dtype)
    w = arrays.ptr(grid.weights, "weights") if grid.weights is not None else None
    _lib.check(_lib.load().sg_evaluate(plan.handle, _lib.i32_array(order),
                                       arrays.ptr(cp, "control_points"), w,
                                       arrays.ptr(ev, "eval"), _lib.stream_handle()))


def evaluate_multi_(grid: SplineGrid, derivative_orders, evals=None, control_points=None):
    """evaluate!(grid; derivative_order = o, eval = evals[i]) for every order o of
    ``derivative_orders`` in one library call that contracts each shared prefix of the
    orders once (e.g. (0,0), (1,0), (0,1): 5 passes instead of 6).  Results are bitwise
    those of separate ``evaluate_`` calls.  ``evals`` defaults to new eval-shaped arrays;
    returns the list of eval arrays."""
    orders = [tuple(int(v) for v in o) for o in derivative_orders]
    for o in orders:
        if len(o) != grid.nin:
            raise ValueError(f"derivative order {o} has {len(o)} entries, the grid {grid.nin}")
        validate_partial_derivatives(grid, o)
    cp = obtain(grid.control_points if control_points is None else control_points)
    assert tuple(cp.shape) == tuple(obtain(grid.control_points).shape)
    if evals is None:
        evals = [arrays.empty(tuple(grid.eval.shape), grid.dtype, grid.eval.device)
                 for _ in orders]
    if len(evals) != len(orders):
        raise ValueError("one eval array per derivative order is needed")
    for ev in evals:
        assert tuple(ev.shape) == tuple(grid.eval.shape)
        if ev.dtype != grid.dtype:
            raise TypeError(f"eval {ev.dtype} does not match the grid's {grid.dtype}")
    if cp.dtype not in (grid.dtype, torch.bfloat16):
        raise TypeError(f"control points {cp.dtype} do not match the grid's {grid.dtype}")
    plan = grid.plan(cp.dtype)
    w = arrays.ptr(grid.weights, "weights") if grid.weights is not None else None
    flat = [v for o in orders for v in o]
    ptrs = (C.c_void_p * max(1, len(evals)))(*[arrays.ptr(ev, "eval") for ev in evals])
    _lib.check(_lib.load().sg_evaluate_multi(plan.handle, len(orders), _lib.i32_array(flat),
                                             arrays.ptr(cp, "control_points"), w, ptrs,
                                             _lib.stream_handle()))
    return evals


def tune_adjoint_(grid: SplineGrid, derivative_order=None, eval=None, control_points=None):
    """Measure and keep the fastest adjoint configuration of the grid's plan (see
    sg_grid_plan_tune); ``eval`` / ``control_points`` serve as scratch (default: the
    grid's eval and a temporary gradient array).  Returns the choice per axis."""
    order = tuple(derivative_order) if derivative_order is not None else (0,) * grid.nin
    validate_partial_derivatives(grid.spline_dimensions, order)
    ev = grid.eval if eval is None else eval
    cp = control_points if control_points is not None else arrays.empty(
        tuple(obtain(grid.control_points).shape), grid.dtype, ev.device)
    return grid.plan(grid.dtype).tune(order, ev, obtain(cp))


def evaluate_adjoint_(grid: SplineGrid, derivative_order=None, control_points=None,
                      eval=None) -> None:
    """evaluate_adjoint!(spline_grid; derivative_order, control_points, eval)
    (src/adjoint.jl:42-83): control_points <- M' * eval.  Deterministic gather form."""
    assert not grid.is_nurbs(), "Adjoint evaluation not supported for NURBS."
    order = tuple(derivative_order) if derivative_order is not None else (0,) * grid.nin
    validate_partial_derivatives(grid.spline_dimensions, order)
    cp = obtain(grid.control_points if control_points is None else control_points)
    ev = grid.eval if eval is None else eval
    assert tuple(cp.shape) == tuple(obtain(grid.control_points).shape)
    assert tuple(ev.shape) == tuple(grid.eval.shape)
    if cp.dtype != grid.dtype or ev.dtype != grid.dtype:
        raise TypeError("adjoint arrays must have the grid's float type")
    plan = grid.plan(grid.dtype)
    _lib.check(_lib.load().sg_evaluate_adjoint(plan.handle, _lib.i32_array(order),
                                               arrays.ptr(ev, "eval"),
                                               arrays.ptr(cp, "control_points"),
                                               _lib.stream_handle()))
