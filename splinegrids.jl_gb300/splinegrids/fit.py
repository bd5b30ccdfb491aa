"""Gradient-descent fits of spline grids with every stage on the device (sg_fit_* of
the C ABI), capturable as one CUDA graph.

The reference's optimisation examples run this loop on the host
(docs/src/examples_optics.md:184-191 and the Optimization.jl call after it): evaluate! of
the orders (0,0), (1,0), (0,1) into three eval arrays, a loss on them, the loss's
gradient with respect to the control points (Enzyme, which calls evaluate_adjoint!,
ext/SplineGridsEnzymeExt.jl) and an optimiser update.  Here a step is

    forward   evaluate_multi_ of the grid's orders   (or GridBatch forward)
    loss      cotangent = w (eval - target), loss = sum w/2 |eval - target|^2   (sg_fit_loss)
    adjoint   evaluate_adjoint_ of each order         (or GridBatch adjoint)
    update    control points -= step * sum of the order gradients               (sg_fit_update)

with fixed arrays, so ``capture()`` records it (or several steps) once and ``replay()``
runs it without host work; a replay gives the bits of the eager steps.  The loss of
every step stays on the device (``loss()`` / ``losses()`` read it).
"""
from __future__ import annotations

import ctypes as C
import weakref

import torch

from . import _lib, arrays
from .control_points import obtain
from .spline_grid import evaluate_adjoint_, evaluate_multi_


class FitLoop:
    """Device-side gradient-descent steps over fixed arrays.

    forward() / adjoint(): callables issuing the library's forward (writing ``evals``)
    and adjoint (reading ``cotangents``, writing ``grads``) on the current stream.
    Terms: ``evals[t]`` against ``targets[t]`` with weight ``weights[t]`` (default 1),
    cotangent written to ``cotangents[t]``.  Parameters: ``params[u]`` (updated in
    place) with ``grads_per_param[u]`` consecutive entries of ``grads``."""

    def __init__(self, forward, adjoint, evals, targets, cotangents, params, grads,
                 grads_per_param, step: float, weights=None):
        if not (len(evals) == len(targets) == len(cotangents)):
            raise ValueError("one target and one cotangent per eval array")
        if len(grads_per_param) != len(params) or sum(grads_per_param) != len(grads):
            raise ValueError("grads_per_param must split grads over params")
        dt = evals[0].dtype
        for t in list(evals) + list(targets) + list(cotangents) + list(params) + list(grads):
            if t.dtype != dt:
                raise TypeError("all arrays of a fit have one dtype")
        for e, t, c in zip(evals, targets, cotangents):
            if e.numel() != t.numel() or e.numel() != c.numel():
                raise ValueError("eval, target and cotangent sizes differ")
        k = 0
        for p, n in zip(params, grads_per_param):
            for g in grads[k:k + n]:
                if g.numel() != p.numel():
                    raise ValueError("a gradient's size differs from its parameter's")
            k += n
        self._forward, self._adjoint = forward, adjoint
        self.evals, self.targets, self.cotangents = list(evals), list(targets), list(cotangents)
        self.params, self.grads = list(params), list(grads)
        self.step_size = float(step)
        nt, npar = len(self.evals), len(self.params)
        ptrs = lambda ts, what: (C.c_void_p * max(1, len(ts)))(*[arrays.ptr(t, what) for t in ts])
        w = None
        if weights is not None:
            w = (C.c_double * nt)(*[float(x) for x in weights])
        h = C.c_void_p()
        lib = _lib.load()
        _lib.check(lib.sg_fit_plan_create(
            arrays.dtype_code(dt), nt, ptrs(self.evals, "eval"), ptrs(self.targets, "target"),
            ptrs(self.cotangents, "cotangent"), (C.c_int64 * max(1, nt))(*[t.numel() for t in self.evals]),
            w, npar, ptrs(self.params, "parameter"),
            (C.c_int64 * max(1, npar))(*[p.numel() for p in self.params]),
            (C.c_int32 * max(1, npar))(*[int(n) for n in grads_per_param]),
            ptrs(self.grads, "gradient"), C.byref(h)))
        self.handle = h
        self._fin = weakref.finalize(self, lib.sg_fit_plan_destroy, h)
        self._graph = None

    def step(self) -> None:
        """One eager step on the current stream (asynchronous)."""
        self._forward()
        _lib.check(_lib.load().sg_fit_loss(self.handle, _lib.stream_handle()))
        self._adjoint()
        _lib.check(_lib.load().sg_fit_update(self.handle, self.step_size, _lib.stream_handle()))

    def capture(self, steps: int = 1) -> None:
        """Record `steps` consecutive steps as one CUDA graph (the library's launches
        only; no step runs while capturing)."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                for _ in range(steps):
                    self.step()
        torch.cuda.current_stream().wait_stream(s)
        self._graph = g

    def replay(self) -> None:
        """Run the captured steps (asynchronous)."""
        if self._graph is None:
            raise RuntimeError("capture() first")
        self._graph.replay()

    def loss(self) -> float:
        """Synchronize and return the loss of the last step."""
        v = C.c_double()
        _lib.check(_lib.load().sg_fit_losses(self.handle, _lib.stream_handle(), C.byref(v), None,
                                             None, 0))
        return v.value

    def losses(self, n: int = 1024) -> list:
        """Synchronize and return the losses of the last min(n, 1024) steps, oldest first."""
        cnt = C.c_int64()
        buf = (C.c_double * n)()
        _lib.check(_lib.load().sg_fit_losses(self.handle, _lib.stream_handle(), None,
                                             C.byref(cnt), buf, n))
        return list(buf[:min(n, cnt.value, 1024)])


def grid_fit(grid, orders, targets, step: float, weights=None, control_points=None) -> FitLoop:
    """A fit of one grid's control points (default: the grid's own) to target arrays of
    the given derivative orders, e.g. orders (0,0), (1,0), (0,1) as in the optics example:
    forward = one evaluate_multi_ call, adjoint = evaluate_adjoint_ per order."""
    orders = [tuple(o) for o in orders]
    cp = obtain(grid.control_points) if control_points is None else control_points
    dt, dev = cp.dtype, cp.device
    shape_e = tuple(grid.eval.shape)
    evals = [arrays.empty(shape_e, dt, dev) for _ in orders]
    cots = [arrays.empty(shape_e, dt, dev) for _ in orders]
    grads = [arrays.empty(tuple(cp.shape), dt, dev) for _ in orders]

    def forward():
        evaluate_multi_(grid, orders, evals=evals, control_points=cp)

    def adjoint():
        for o, c, g in zip(orders, cots, grads):
            evaluate_adjoint_(grid, derivative_order=o, eval=c, control_points=g)

    return FitLoop(forward, adjoint, evals, list(targets), cots, [cp], grads, [len(orders)], step,
                   weights)


def batch_fit(batch, targets, step: float, weights=None) -> FitLoop:
    """A fit of every grid of a GridBatch (its set arrays: control points, evals,
    cotangents, gradients) to one target per grid, with the batch's forward and adjoint
    launches around the loss."""
    cps, evals, cots, grads = batch._arrays
    if any(a is None for a in (cps, evals, cots, grads)):
        raise ValueError("the batch needs all four arrays set (GridBatch.set_arrays)")
    cps = [obtain(c) for c in cps]
    return FitLoop(lambda: batch.run(forward=True, adjoint=False),
                   lambda: batch.run(forward=False, adjoint=True),
                   evals, list(targets), cots, cps, grads, [1] * len(cps), step, weights)
