"""A spline grid as a linear map, and its least-squares fit on the device.

``LinearMap(spline_grid; derivative_order)`` mirrors the reference's LinearMaps extension
(ext/SplineGridsLinearMapsExt.jl:5-52): the map takes the flat control-point unknowns
(``get_n_control_points(grid) * Nout`` values, [n_control_points, Nout] column-major)
to the flat eval array; forward = copyto!(control_points, x); evaluate!(control_points);
evaluate!(grid; derivative_order, eval = y), adjoint = evaluate_adjoint!(grid;
derivative_order, eval = y); evaluate_adjoint!(control_points); copyto!(x,
control_points).  As in the reference, both directions use the grid's control points as
their working storage.

``lsqr(A, b)`` solves min ||A x - b|| as the reference's fits do with IterativeSolvers'
``lsqr`` (test/test_LinearMapsExt.jl:14-61), with the library's device LSQR: all vectors
and scalars stay on the GPU, and by default one iteration is captured once into a CUDA
graph whose device-side while loop runs the whole solve in one launch.
"""
from __future__ import annotations

import ctypes as C
import math
import weakref

import torch

from . import _lib, arrays
from .control_points import (LocallyRefinedControlPoints,
                             evaluate_adjoint_control_points_, evaluate_control_points_,
                             get_n_control_points, obtain)
from .spline_grid import (SplineGrid, evaluate_, evaluate_adjoint_, validate_partial_derivatives)


def _copy_in(control_points, x: torch.Tensor) -> None:
    """copyto!(control_points, reshape(x, n_control_points, Nout)), without allocating."""
    if isinstance(control_points, LocallyRefinedControlPoints):
        ncp, nout = control_points.n_control_points(), control_points.nout
        xm = arrays.reshape(x, (ncp, nout))
        r = 0
        for lr in control_points.local_refinements:
            n = lr.n_refined
            lr.refinement_values.copy_(xm[r:r + n])
            r += n
    else:
        arrays.vec(obtain(control_points)).copy_(x)


def _copy_out(x: torch.Tensor, control_points) -> None:
    """copyto!(reshape(x, n_control_points, Nout), control_points), without allocating."""
    if isinstance(control_points, LocallyRefinedControlPoints):
        ncp, nout = control_points.n_control_points(), control_points.nout
        xm = arrays.reshape(x, (ncp, nout))
        r = 0
        for lr in control_points.local_refinements:
            n = lr.n_refined
            xm[r:r + n].copy_(lr.refinement_values)
            r += n
    else:
        x.copy_(arrays.vec(obtain(control_points)))


class LinearMap:
    """LinearMap(spline_grid; derivative_order) of the reference's extension: an
    ``m x n`` operator, m = numel(eval), n = get_n_control_points(grid) * Nout, acting on
    flat (1-D, contiguous) CUDA tensors of the grid's float type."""

    def __init__(self, spline_grid: SplineGrid, derivative_order=None):
        order = tuple(derivative_order) if derivative_order is not None else \
            (0,) * spline_grid.nin
        validate_partial_derivatives(spline_grid, order)
        self.grid = spline_grid
        self.derivative_order = order
        self.shape = (spline_grid.eval.numel(),
                      get_n_control_points(spline_grid) * spline_grid.nout)
        self.dtype = spline_grid.dtype
        self.device = spline_grid.eval.device

    def _check(self, t: torch.Tensor, length: int, what: str) -> None:
        if t.dim() != 1 or t.numel() != length or not t.is_contiguous():
            raise ValueError(f"{what} must be a contiguous 1-D tensor of length {length}")
        if t.dtype != self.dtype or t.device != self.device:
            raise TypeError(f"{what} must be {self.dtype} on {self.device}")

    def mul_(self, y: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
        """mul!(y, A, x): y = A x (the extension's forward closure)."""
        self._check(y, self.shape[0], "y")
        self._check(x, self.shape[1], "x")
        g = self.grid
        _copy_in(g.control_points, x)
        evaluate_control_points_(g.control_points)
        evaluate_(g, self.derivative_order, eval=arrays.reshape(y, tuple(g.eval.shape)))
        return y

    def rmul_(self, x: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
        """mul!(x, A', y): x = A' y (the extension's adjoint closure)."""
        self._check(y, self.shape[0], "y")
        self._check(x, self.shape[1], "x")
        g = self.grid
        evaluate_adjoint_(g, self.derivative_order, eval=arrays.reshape(y, tuple(g.eval.shape)))
        evaluate_adjoint_control_points_(g.control_points)
        _copy_out(x, g.control_points)
        return x

    def __matmul__(self, x: torch.Tensor) -> torch.Tensor:
        y = torch.empty(self.shape[0], dtype=self.dtype, device=self.device)
        return self.mul_(y, x)

    @property
    def T(self) -> "_Adjoint":
        return _Adjoint(self)

    def adjoint(self) -> "_Adjoint":
        return _Adjoint(self)

    def __repr__(self):
        return f"{self.shape[0]}x{self.shape[1]} LinearMap of a {self.grid!r}"


class _Adjoint:
    def __init__(self, A: LinearMap):
        self.A = A
        self.shape = (A.shape[1], A.shape[0])

    def __matmul__(self, y: torch.Tensor) -> torch.Tensor:
        x = torch.empty(self.A.shape[1], dtype=self.A.dtype, device=self.A.device)
        return self.A.rmul_(x, y)


ISTOP = {
    -1: "non-finite values in the recurrence",
    0: "x = 0 is the exact solution",
    1: "A x = b solved to btol / atol",
    2: "least-squares solution to atol",
    3: "cond(A) estimate exceeds conlim",
    4: "A x = b solved to machine precision",
    5: "least-squares solution to machine precision",
    6: "cond(A) estimate too large for the working precision",
    7: "maxiter reached",
}


class LSQRSolver:
    """Device LSQR for one LinearMap, reusable across right-hand sides.

    Construction allocates the solver's vectors (U, F of length m; V, W, X, G of length
    n), applies A and A' once so that every plan the operator needs exists, and (with
    ``graph=True``) captures the solve: prologue, then one iteration as the body of a
    device-side while loop.  ``solve(b)`` then copies b into the solver's buffer and
    launches the graph once; the host waits only when it reads the result.  Defaults
    follow IterativeSolvers' lsqr: atol = btol = sqrt(eps), conlim = 1/sqrt(eps),
    maxiter = max(m, n)."""

    def __init__(self, A: LinearMap, *, damp: float = 0.0, atol=None, btol=None, conlim=None,
                 maxiter=None, graph: bool = True):
        self.A = A
        m, n = A.shape
        eps = torch.finfo(A.dtype).eps
        atol = math.sqrt(eps) if atol is None else float(atol)
        btol = math.sqrt(eps) if btol is None else float(btol)
        conlim = 1.0 / math.sqrt(eps) if conlim is None else float(conlim)
        maxiter = max(m, n) if maxiter is None else int(maxiter)
        mk = lambda k: torch.zeros(k, dtype=A.dtype, device=A.device)
        self.B, self.U, self.F = mk(m), mk(m), mk(m)
        self.V, self.W, self.X, self.G = mk(n), mk(n), mk(n), mk(n)
        lib = _lib.load()
        h = C.c_void_p()
        _lib.check(lib.sg_lsqr_create(arrays.dtype_code(A.dtype), m, n, self.U.data_ptr(),
                                      self.V.data_ptr(), self.W.data_ptr(), self.X.data_ptr(),
                                      self.F.data_ptr(), self.G.data_ptr(), float(damp), atol,
                                      btol, conlim, maxiter, C.byref(h)))
        self.handle = h
        self._fin = weakref.finalize(self, lib.sg_lsqr_destroy, h)
        # create every plan and device table the operator uses before any capture
        A.mul_(self.F, self.V)
        A.rmul_(self.G, self.U)
        self.graph = False
        if graph:
            self._capture()
            self.graph = True

    # --------------------------------------------------------------- steps
    def _prologue(self, s: int) -> None:
        lib = _lib.load()
        _lib.check(lib.sg_lsqr_start(self.handle, self.B.data_ptr(), s))
        self.A.rmul_(self.G, self.U)
        _lib.check(lib.sg_lsqr_after_adjoint(self.handle, s))

    def _iteration(self, s: int) -> None:
        lib = _lib.load()
        self.A.mul_(self.F, self.V)
        _lib.check(lib.sg_lsqr_after_forward(self.handle, s))
        self.A.rmul_(self.G, self.U)
        _lib.check(lib.sg_lsqr_after_adjoint(self.handle, s))

    def _capture(self) -> None:
        lib = _lib.load()
        # stream capture needs a created stream (the legacy default stream cannot capture)
        cs = torch.cuda.Stream(device=self.A.device)
        cs.wait_stream(torch.cuda.current_stream(self.A.device))
        with torch.cuda.stream(cs):
            s = _lib.stream_handle()
            _lib.check(lib.sg_lsqr_capture_begin(self.handle, s))
            try:
                self._prologue(s)
                body = C.c_void_p()
                _lib.check(lib.sg_lsqr_capture_body(self.handle, s, C.byref(body)))
                bs = torch.cuda.ExternalStream(body.value, device=self.A.device)
                with torch.cuda.stream(bs):
                    self._iteration(_lib.stream_handle())
            finally:
                _lib.check(lib.sg_lsqr_capture_end(self.handle, s))
        torch.cuda.current_stream(self.A.device).wait_stream(cs)

    def info(self) -> dict:
        """Iterations, stop code and the solver's norm estimates (synchronizes)."""
        counts = (C.c_int64 * 3)()
        norms = (C.c_double * 6)()
        _lib.check(_lib.load().sg_lsqr_info(self.handle, _lib.stream_handle(), counts, norms))
        keys = ("anorm", "acond", "rnorm", "arnorm", "xnorm", "bnorm")
        d = dict(iterations=int(counts[0]), istop=int(counts[1]), done=bool(counts[2]))
        d.update({k: float(norms[i]) for i, k in enumerate(keys)})
        d["reason"] = ISTOP.get(d["istop"], "unknown")
        return d

    def solve(self, b: torch.Tensor, x: torch.Tensor | None = None) -> torch.Tensor:
        """x = argmin ||A x - b|| from x0 = 0; returns x (a new tensor unless given).
        ``b`` is the flat eval vector or an eval-shaped column-major array."""
        if b.dim() != 1:
            b = arrays.vec(b)
        self.A._check(b, self.A.shape[0], "b")
        self.B.copy_(b)
        lib = _lib.load()
        s = _lib.stream_handle()
        if self.graph:
            _lib.check(lib.sg_lsqr_launch(self.handle, s))
        else:
            self._prologue(s)
            while not self.info()["done"]:
                self._iteration(s)
        out = x if x is not None else torch.empty_like(self.X)
        out.copy_(self.X)
        return out


def lsqr(A: LinearMap, b: torch.Tensor, *, damp: float = 0.0, atol=None, btol=None,
         conlim=None, maxiter=None, graph: bool = True, log: bool = False):
    """IterativeSolvers-style ``lsqr(A, b)`` on the device: returns x (and, with
    ``log=True``, the solver's info dict as a second value)."""
    solver = LSQRSolver(A, damp=damp, atol=atol, btol=btol, conlim=conlim, maxiter=maxiter,
                        graph=graph)
    x = solver.solve(b)
    return (x, solver.info()) if log else x
