"""Many grids in one persistent launch (sg_batch_* of the C ABI).

The reference evaluates one grid per `evaluate!` / `evaluate_adjoint!` call.  A
``GridBatch`` holds any number of non-NURBS grids of degree <= 3 (sizes, degrees and
channel counts may all differ) and runs all their forward and/or adjoint work in a few
launches: 2D grids on the fused path (both axes per unit of work; forward tiles in one
launch, adjoint tiles in one persistent launch fed by a device-side work queue), the
others through the separable passes in one persistent launch fed by a device-side work
queue; per grid the results equal
``evaluate_`` / ``evaluate_adjoint_``.  Control-point sets are folded into the channel
axis (Nout), the slowest index of control points and eval.
"""
from __future__ import annotations

import ctypes as C
import weakref

import torch

from . import _lib, arrays
from .control_points import obtain
from .spline_grid import SplineGrid, validate_partial_derivatives

FORWARD = 1
ADJOINT = 2


class GridBatch:
    def __init__(self, grids, derivative_orders=None):
        self.grids = list(grids)
        n = len(self.grids)
        if n == 0:
            raise ValueError("GridBatch needs at least one grid")
        orders = derivative_orders or [(0,) * g.nin for g in self.grids]
        descs = (_lib.GridDesc * n)()
        ords = (C.c_int32 * (n * _lib.SG_MAX_NIN))()
        self._keep = []
        for gi, (g, o) in enumerate(zip(self.grids, orders)):
            if not isinstance(g, SplineGrid) or g.is_nurbs():
                raise TypeError("GridBatch takes non-NURBS SplineGrids")
            validate_partial_derivatives(g, tuple(o))
            d = descs[gi]
            d.nin, d.nout, d.dtype, d.has_weights = g.nin, g.nout, arrays.dtype_code(g.dtype), 0
            for k, sd in enumerate(g.spline_dimensions):
                d.n_samples[k] = len(sd)
                d.n_basis[k] = sd.n_basis_functions
                d.degree[k] = sd.degree
                d.max_derivative_order[k] = sd.max_derivative_order
                d.sample_indices[k] = sd.sample_indices.data_ptr()
                d.basis_eval[k] = arrays.ptr(sd.eval, "basis table")
                ords[gi * _lib.SG_MAX_NIN + k] = int(o[k])
        h = C.c_void_p()
        lib = _lib.load()
        _lib.check(lib.sg_batch_plan_create(n, descs, ords, _lib.stream_handle(), C.byref(h)))
        self.handle = h
        self._fin = weakref.finalize(self, lib.sg_batch_plan_destroy, h)
        self.orders = [tuple(o) for o in orders]

    def set_arrays(self, control_points=None, evals=None, eval_bars=None,
                   control_points_bars=None) -> None:
        """Per grid: control points / eval (forward), cotangent / gradient (adjoint);
        lists of column-major CUDA tensors, or None for an unused pair."""
        n = len(self.grids)

        def table(ts, what):
            if ts is None:
                return None
            assert len(ts) == n, f"{what}: one tensor per grid"
            arr = (C.c_void_p * n)()
            for i, t in enumerate(ts):
                arr[i] = arrays.ptr(obtain(t), what)
            return arr

        for g, cp, ev in zip(self.grids, control_points or [None] * n, evals or [None] * n):
            if cp is not None:
                assert tuple(obtain(cp).shape) == tuple(obtain(g.control_points).shape)
            if ev is not None:
                assert tuple(ev.shape) == tuple(g.eval.shape)
        self._arrays = (control_points, evals, eval_bars, control_points_bars)
        _lib.check(_lib.load().sg_batch_set_arrays(
            self.handle, table(control_points, "control points"), table(evals, "eval"),
            table(eval_bars, "eval_bar"), table(control_points_bars, "control_points_bar")))

    def run(self, forward: bool = True, adjoint: bool = False) -> None:
        """One launch over every grid (asynchronous; capturable in a CUDA graph)."""
        what = (FORWARD if forward else 0) | (ADJOINT if adjoint else 0)
        _lib.check(_lib.load().sg_batch_run(self.handle, what, _lib.stream_handle()))

    def set_strategy(self, strategy: str) -> None:
        """"auto" (every grid that fits runs fused: Nin = 2, both axes per unit of work,
        no intermediates) or "separable" (every grid in the dependency-ordered pass
        queue); results are bitwise the same.  Rebuilds the work lists."""
        code = {"auto": 0, "separable": 1, "fused": 2}[strategy]
        _lib.check(_lib.load().sg_batch_set_strategy(self.handle, code))

    def tune(self) -> tuple:
        """Time candidate sizes of the fused forward units and adjoint tiles on the set
        arrays (eval and gradients are overwritten) and keep the fastest; returns
        (forward values per unit, adjoint values per tile, 0 = axis 1 whole).  Results
        are bitwise the same for every size."""
        out = (C.c_int64 * 2)()
        _lib.check(_lib.load().sg_batch_tune(self.handle, _lib.stream_handle(), out))
        return int(out[0]), int(out[1])

    def set_unit_sizes(self, forward_values: int = 0, adjoint_values: int = 0) -> None:
        """Explicit fused unit sizes (0: the built-in ones)."""
        _lib.check(_lib.load().sg_batch_set_unit_sizes(self.handle, int(forward_values),
                                                         int(adjoint_values)))

    def fused_grids(self) -> int:
        """Grids on the fused path."""
        return int(_lib.load().sg_batch_fused_grids(self.handle))

    def check(self) -> None:
        """Synchronize and raise if a device-side dependency wait of the last run timed out."""
        _lib.check(_lib.load().sg_batch_check(self.handle, _lib.stream_handle()))

    PASS_KINDS = ("forward axis 0", "forward axis >= 1", "adjoint axis >= 1 (warp tasks)",
                  "adjoint axis 0", "adjoint axis >= 1 (bulk-copy stream)")

    def enable_profile(self, on: bool = True) -> None:
        """Count SM cycles per pass kind in later runs (see profile())."""
        _lib.check(_lib.load().sg_batch_enable_profile(self.handle, 1 if on else 0))

    def profile(self) -> dict:
        """Synchronize and return {kind: (wait_cycles, work_cycles, items)} since the
        last call, then clear the counters."""
        out = (C.c_int64 * 15)()
        _lib.check(_lib.load().sg_batch_profile(self.handle, _lib.stream_handle(), out))
        return {k: (int(out[3 * i]), int(out[3 * i + 1]), int(out[3 * i + 2]))
                for i, k in enumerate(self.PASS_KINDS)}

    def workspace_bytes(self) -> int:
        return int(_lib.load().sg_batch_plan_workspace_bytes(self.handle))

    def items(self, forward=True, adjoint=False) -> int:
        what = (FORWARD if forward else 0) | (ADJOINT if adjoint else 0)
        return int(_lib.load().sg_batch_items(self.handle, what))


def chunk_ranges(sizes, n_chunks: int):
    """Consecutive [a, b) ranges of items cut where the running size passes k/n_chunks of
    the total (about equal output per chunk; at most n_chunks, none empty)."""
    n = len(sizes)
    n_chunks = max(1, min(int(n_chunks), n))
    total = float(sum(sizes))
    bounds, acc, k = [0], 0.0, 1
    for i, sz in enumerate(sizes):
        acc += sz
        if k < n_chunks and acc >= total * k / n_chunks and i + 1 < n:
            bounds.append(i + 1)
            k += 1
    bounds.append(n)
    return [(a, b) for a, b in zip(bounds[:-1], bounds[1:]) if b > a]


class GridBatchPipeline:
    """Forward and/or adjoint of many grids with host inputs and outputs, the transfers
    overlapped with the compute.

    The grids are cut into ``n_chunks`` consecutive sub-batches of about equal output
    size, each a ``GridBatch`` (one persistent launch).  Per call, chunk k's inputs
    (control points, cotangents) go host -> device on one copy stream, its launch runs on
    the caller's stream once they have landed, and its outputs (eval, gradients) go
    device -> host on a second copy stream, so chunk k+1's uploads and chunk k-1's
    downloads overlap chunk k's launch and each other (the host link carries both
    directions at once).  Per grid the results are those of ``GridBatch.run``.

    Device arrays are the caller's (per grid, as ``GridBatch.set_arrays``); host arrays
    should be pinned (page-locked) for the copies to be asynchronous."""

    def __init__(self, grids, control_points=None, evals=None, eval_bars=None,
                 control_points_bars=None, n_chunks: int = 8):
        grids = list(grids)
        self.ranges = chunk_ranges([g.eval.numel() for g in grids], n_chunks)
        pick = lambda ts, a, b: None if ts is None else list(ts[a:b])
        self.batches = []
        for a, b in self.ranges:
            bt = GridBatch(grids[a:b])
            bt.set_arrays(pick(control_points, a, b), pick(evals, a, b), pick(eval_bars, a, b),
                          pick(control_points_bars, a, b))
            self.batches.append(bt)
        self.device_arrays = (control_points, evals, eval_bars, control_points_bars)
        dev = grids[0].eval.device
        self.s_in = torch.cuda.Stream(device=dev)
        self.s_out = torch.cuda.Stream(device=dev)
        self._graph = None       # capture(): the recorded step
        self._graph_host = []    # and the host arrays its copies read and write

    def run(self, h_control_points=None, h_evals=None, h_eval_bars=None,
            h_control_points_bars=None, forward: bool = True, adjoint: bool = True) -> None:
        """Upload h_control_points / h_eval_bars, run, download into h_evals /
        h_control_points_bars (per grid host tensors in the device arrays' layout; None
        skips a direction).  Asynchronous with respect to the host."""
        d_cp, d_ev, d_cot, d_gr = self.device_arrays
        lib = _lib.load()

        def pairs(dsts, srcs, a, b):
            out = []
            for i in range(a, b):
                dst, src = obtain(dsts[i]), obtain(srcs[i])
                if tuple(dst.shape) != tuple(src.shape) or dst.dtype != src.dtype:
                    raise ValueError(f"grid {i}: host and device arrays differ in shape or type")
                if not (arrays.is_colmajor(dst) and arrays.is_colmajor(src)):
                    raise ValueError(f"grid {i}: arrays must be column-major (Julia layout)")
                out.append((dst.data_ptr(), src.data_ptr(), dst.numel() * dst.element_size()))
            return out

        def issue(entries, stream):  # one library call per direction and chunk
            n = len(entries)
            if n == 0:
                return
            dst = (C.c_void_p * n)(*[e[0] for e in entries])
            src = (C.c_void_p * n)(*[e[1] for e in entries])
            nb = (C.c_int64 * n)(*[e[2] for e in entries])
            _lib.check(lib.sg_copy_list(n, dst, src, nb, stream.cuda_stream))

        cur = torch.cuda.current_stream()
        self.s_in.wait_stream(cur)   # the previous call's launches have read their inputs
        self.s_out.wait_stream(cur)
        for bt, (a, b) in zip(self.batches, self.ranges):
            ups = []
            if forward and h_control_points is not None:
                ups += pairs(d_cp, h_control_points, a, b)
            if adjoint and h_eval_bars is not None:
                ups += pairs(d_cot, h_eval_bars, a, b)
            issue(ups, self.s_in)
            landed = torch.cuda.Event()
            landed.record(self.s_in)
            cur.wait_event(landed)
            bt.run(forward=forward, adjoint=adjoint)
            done = torch.cuda.Event()
            done.record(cur)
            self.s_out.wait_event(done)
            downs = []
            if forward and h_evals is not None:
                downs += pairs(h_evals, d_ev, a, b)
            if adjoint and h_control_points_bars is not None:
                downs += pairs(h_control_points_bars, d_gr, a, b)
            issue(downs, self.s_out)
        cur.wait_stream(self.s_out)
        cur.wait_stream(self.s_in)

    def capture(self, h_control_points=None, h_evals=None, h_eval_bars=None,
                h_control_points_bars=None, forward: bool = True, adjoint: bool = True) -> None:
        """Record one ``run`` with these host arrays as a CUDA graph: every upload,
        sub-batch launch and download, with the same stream overlap.  ``replay()`` then
        repeats the whole step with one launch, so the host issues no per-array work and
        a pause of the host thread does not leave the GPU idle.  The graph copies from and
        to the host arrays' memory when it runs: new contents of the same arrays are
        picked up, and the arrays must stay alive (they are kept referenced) and pinned.
        No step runs while capturing."""
        host = [h for hs in (h_control_points, h_evals, h_eval_bars, h_control_points_bars)
                if hs is not None for h in hs]
        for i, h in enumerate(host):
            if not obtain(h).is_pinned():
                raise ValueError(f"host array {i} is not pinned: a captured copy needs page-locked memory")
        cur = torch.cuda.current_stream()
        s = torch.cuda.Stream(device=cur.device)
        s.wait_stream(cur)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.run(h_control_points, h_evals, h_eval_bars, h_control_points_bars,
                         forward=forward, adjoint=adjoint)
        cur.wait_stream(s)
        self._graph = g
        self._graph_host = host

    def replay(self) -> None:
        """Run the captured step (asynchronous with respect to the host)."""
        if self._graph is None:
            raise RuntimeError("capture() first")
        self._graph.replay()

    def check(self) -> None:
        for bt in self.batches:
            bt.check()
