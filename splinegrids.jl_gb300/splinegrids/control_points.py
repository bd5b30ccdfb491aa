"""Control-point containers and the refinement application
(src/control_points.jl:1-356, src/adjoint.jl:85-205, src/refinement_matrix.jl:405-445).

``mult_`` / ``mult_adjoint_`` and the local-refinement overwrite (and its adjoint) run on
the device through the library; the bookkeeping of LocalRefinement levels is host
logic, as in the reference.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib, arrays


def _stream():
    return _lib.stream_handle()


class DefaultControlPoints:
    """A thin wrapper around a control-point array [n_basis..., Nout]
    (src/control_points.jl:1-57)."""

    def __init__(self, control_points: torch.Tensor):
        self.control_points = control_points

    @property
    def nin(self):
        return self.control_points.dim() - 1

    @property
    def nout(self):
        return self.control_points.shape[-1]

    @property
    def shape(self):
        return tuple(self.control_points.shape)

    def size(self):
        return self.shape

    @property
    def dtype(self):
        return self.control_points.dtype

    def n_control_points(self) -> int:
        return math.prod(self.shape[:-1])

    def copy_(self, vals) -> None:
        """copyto!(control_points, vals): vals shaped like the array or as
        [n_control_points, Nout]."""
        v = torch.as_tensor(vals, device=self.control_points.device)
        if tuple(v.shape) != self.shape:
            v = arrays.reshape(arrays.vec(v.to(self.dtype)), self.shape)
        self.control_points.copy_(v)

    def values_matrix(self) -> torch.Tensor:
        """The [n_control_points, Nout] view used by copyto!(M, control_points)."""
        return arrays.reshape(arrays.vec(self.control_points), (self.n_control_points(), self.nout))

    def __repr__(self):
        return (f"DefaultControlPoints for grid of size {self.shape[:-1]} in R^{self.nout} "
                f"({self.dtype}).")


class LocalRefinement:
    """One level of a locally refined hierarchy (src/control_points.jl:59-154): the
    refinement matrices along ``dims_refinement`` (0-based) and the control points
    overwritten after applying them (1-based ``refinement_indices`` [n, Nin],
    ``refinement_values`` [n, Nout], device tensors)."""

    def __init__(self, dims_refinement, refinement_matrices, refinement_indices: torch.Tensor,
                 refinement_values: torch.Tensor):
        self.dims_refinement = [int(d) for d in dims_refinement]
        self.refinement_matrices = list(refinement_matrices)
        self.refinement_indices = refinement_indices
        self.refinement_values = refinement_values

    @property
    def n_refined(self) -> int:
        return int(self.refinement_indices.shape[0])


class LocallyRefinedControlPoints:
    """Control points of a truncated hierarchical basis (THB) spline
    (src/control_points.jl:156-198): ``control_points_refined[i]`` is the dense grid of
    level i; ``obtain`` gives the finest level."""

    def __init__(self, control_points_refined, local_refinements):
        self.control_points_refined = list(control_points_refined)
        self.local_refinements = list(local_refinements)

    @property
    def nin(self):
        return self.control_points_refined[0].dim() - 1

    @property
    def nout(self):
        return self.control_points_refined[0].shape[-1]

    @property
    def shape(self):
        return tuple(self.control_points_refined[-1].shape)

    def size(self):
        return self.shape

    @property
    def dtype(self):
        return self.control_points_refined[0].dtype

    def n_control_points(self) -> int:
        """get_n_control_points (src/control_points.jl:283-290)."""
        return sum(lr.n_refined for lr in self.local_refinements)

    def values_matrix(self) -> torch.Tensor:
        """vcat of the refinement values of all levels (get_control_point_view,
        src/control_points.jl:200-208), as a new [n_control_points, Nout] tensor."""
        return torch.cat([lr.refinement_values for lr in self.local_refinements], 0)

    def copy_(self, vals) -> None:
        """copyto!(control_points, M): scatter rows of M into the levels' values."""
        v = torch.as_tensor(vals, device=self.local_refinements[0].refinement_values.device)
        v = arrays.reshape(arrays.vec(v.to(self.dtype)), (self.n_control_points(), self.nout))
        r = 0
        for lr in self.local_refinements:
            n = lr.n_refined
            lr.refinement_values.copy_(v[r:r + n])
            r += n

    def __repr__(self):
        return (f"LocallyRefinedControlPoints for final grid of size {self.shape[:-1]} in "
                f"R^{self.nout} ({self.dtype}). Local refinements: {len(self.local_refinements)}")


def obtain(control_points):
    """obtain (src/control_points.jl:351-356)."""
    if isinstance(control_points, DefaultControlPoints):
        return control_points.control_points
    if isinstance(control_points, LocallyRefinedControlPoints):
        return control_points.control_points_refined[-1]
    return control_points


def get_n_control_points(obj) -> int:
    cp = getattr(obj, "control_points", obj)
    if isinstance(cp, (DefaultControlPoints, LocallyRefinedControlPoints)):
        return cp.n_control_points()
    return math.prod(tuple(cp.shape)[:-1])


# ---------------------------------------------------------------------- device ops
def _refmat_structs(As, device, dtype):
    arr = (_lib.RefMat * max(1, len(As)))()
    keep = []
    for r, A in enumerate(As):
        rp, cs, nz = A.device_arrays(device, dtype)
        keep += [rp, cs, nz]
        arr[r].m, arr[r].n, arr[r].nnz = A.m, A.n, len(A.nzval)
        arr[r].row_pointer, arr[r].column_start, arr[r].nzval = (rp.data_ptr(), cs.data_ptr(),
                                                                  nz.data_ptr())
    return arr, keep


def mult_(Y: torch.Tensor, As, B: torch.Tensor, dims_refinement) -> None:
    """mult!(Y, As, B, dims_refinement) (src/refinement_matrix.jl:405-445): left-multiply
    B by each refinement matrix along its (0-based) dimension, into Y."""
    arr, keep = _refmat_structs(As, B.device, B.dtype)
    _lib.check(_lib.load().sg_mult(
        arrays.dtype_code(B.dtype), B.dim(), _lib.i64_array(Y.shape), _lib.i64_array(B.shape),
        len(As), arr, _lib.i32_array(dims_refinement), arrays.ptr(B, "B"), arrays.ptr(Y, "Y"),
        _stream()))
    del keep


def mult_adjoint_(B: torch.Tensor, As, Y: torch.Tensor, dims_refinement) -> None:
    """mult_adjoint!(B, As, Y, dims_refinement) (src/adjoint.jl:127-152); overwrites B."""
    arr, keep = _refmat_structs(As, Y.device, Y.dtype)
    _lib.check(_lib.load().sg_mult_adjoint(
        arrays.dtype_code(Y.dtype), Y.dim(), _lib.i64_array(Y.shape), _lib.i64_array(B.shape),
        len(As), arr, _lib.i32_array(dims_refinement), arrays.ptr(Y, "Y"), arrays.ptr(B, "B"),
        _stream()))
    del keep


def local_refinement_(cp: torch.Tensor, refinement_indices: torch.Tensor,
                      refinement_values: torch.Tensor) -> None:
    """local_refinement_kernel (src/control_points.jl:296-311)."""
    n = int(refinement_indices.shape[0])
    if n == 0:
        return
    _lib.check(_lib.load().sg_local_refinement(
        arrays.dtype_code(cp.dtype), cp.dim() - 1, cp.shape[-1], _lib.i64_array(cp.shape[:-1]), n,
        arrays.ptr(refinement_indices, "refinement_indices"),
        arrays.ptr(refinement_values, "refinement_values"), arrays.ptr(cp, "control_points"),
        _stream()))


def local_refinement_adjoint_(refinement_values: torch.Tensor, cp: torch.Tensor,
                              refinement_indices: torch.Tensor) -> None:
    """local_refinement_adjoint_kernel (src/adjoint.jl:154-170)."""
    n = int(refinement_indices.shape[0])
    if n == 0:
        return
    _lib.check(_lib.load().sg_local_refinement_adjoint(
        arrays.dtype_code(cp.dtype), cp.dim() - 1, cp.shape[-1], _lib.i64_array(cp.shape[:-1]), n,
        arrays.ptr(refinement_indices, "refinement_indices"),
        arrays.ptr(refinement_values, "refinement_values"), arrays.ptr(cp, "control_points"),
        _stream()))


def evaluate_control_points_(control_points) -> None:
    """evaluate!(::LocallyRefinedControlPoints) (src/control_points.jl:313-349): per level,
    apply the refinement matrices then overwrite the activated control points.  A no-op
    for DefaultControlPoints."""
    if not isinstance(control_points, LocallyRefinedControlPoints):
        return
    cps, lrs = control_points.control_points_refined, control_points.local_refinements
    for i, lr in enumerate(lrs):
        if i > 0:
            mult_(cps[i], lr.refinement_matrices, cps[i - 1], lr.dims_refinement)
        local_refinement_(cps[i], lr.refinement_indices, lr.refinement_values)


def evaluate_adjoint_control_points_(control_points) -> None:
    """evaluate_adjoint!(::LocallyRefinedControlPoints) (src/adjoint.jl:172-205): in reverse
    over the levels, gather-and-zero the overwritten entries into the refinement values,
    then apply the adjoint refinement into the previous level."""
    if not isinstance(control_points, LocallyRefinedControlPoints):
        return
    cps, lrs = control_points.control_points_refined, control_points.local_refinements
    for i in range(len(lrs) - 1, -1, -1):
        lr = lrs[i]
        local_refinement_adjoint_(lr.refinement_values, cps[i], lr.refinement_indices)
        if i > 0:
            mult_adjoint_(cps[i - 1], lr.refinement_matrices, cps[i], lr.dims_refinement)


def cartesian_indices(shape) -> np.ndarray:
    """1-based CartesianIndices of `shape` in column-major order as an [n, ndims] array
    (collect_indices, src/utils.jl:187-196)."""
    grids = np.meshgrid(*[np.arange(1, s + 1) for s in shape], indexing="ij")
    return np.stack([g.flatten(order="F") for g in grids], axis=1).astype(np.int32)


def index_tensor(idx_np: np.ndarray, device) -> torch.Tensor:
    """[n, Nin] 1-based int32 indices as a column-major device tensor."""
    idx_np = np.asarray(idx_np, dtype=np.int32).reshape(-1, idx_np.shape[1] if idx_np.ndim == 2
                                                         else 1)
    return arrays.from_any(torch.as_tensor(idx_np), torch.int32, device)


def _unique_rows_stable(a: np.ndarray) -> np.ndarray:
    """unique(A; dims=1): first occurrences, in order."""
    seen, keep = set(), []
    for i, row in enumerate(map(tuple, a)):
        if row not in seen:
            seen.add(row)
            keep.append(i)
    return a[keep] if len(keep) else a[:0]


def activate_local_refinement_(control_points: LocallyRefinedControlPoints, refinement_indices,
                               refinement_index: int | None = None) -> None:
    """activate_local_refinement! (src/control_points.jl:458-516): append the given 1-based
    indices (unique rows) to a level's overwritten control points, with values read from
    that level's current control-point grid so the geometry does not change."""
    lrs = control_points.local_refinements
    level = len(lrs) - 1 if refinement_index is None else int(refinement_index)
    lr = lrs[level]
    cp_level = control_points.control_points_refined[level]
    nin, nout = cp_level.dim() - 1, cp_level.shape[-1]
    new = np.asarray(refinement_indices, dtype=np.int32).reshape(-1, nin)
    assert new.shape[1] == nin, \
        "Number of indices per control point must match the number of input dimensions."
    old = lr.refinement_indices.cpu().numpy()
    allidx = _unique_rows_stable(np.concatenate([old.reshape(-1, nin), new], 0))
    n_old = old.shape[0]
    vals = arrays.empty((allidx.shape[0], nout), cp_level.dtype, cp_level.device)
    if n_old:
        vals[:n_old].copy_(lr.refinement_values)
    if allidx.shape[0] > n_old:
        add = allidx[n_old:] - 1
        if np.any(add < 0) or np.any(add >= np.asarray(cp_level.shape[:-1])):
            raise IndexError("refinement index outside the control-point grid")
        sel = tuple(torch.as_tensor(add[:, d], device=cp_level.device, dtype=torch.long)
                    for d in range(nin))
        vals[n_old:].copy_(cp_level[sel])
    lrs[level] = LocalRefinement(lr.dims_refinement, lr.refinement_matrices,
                                 index_tensor(allidx, cp_level.device), vals)


def _workspace(n: int, device) -> torch.Tensor:
    nb = int(_lib.load().sg_select_workspace_bytes(int(n)))
    return torch.empty(max(nb, 16), dtype=torch.uint8, device=device)


def deactivate_overwritten_control_points_(control_points: LocallyRefinedControlPoints,
                                           level: int | None = None) -> None:
    """deactivate_overwritten_control_points! (src/control_points.jl:580-680): drop the
    overwritten control points of a level whose effect is completely overwritten at the
    next level.  As in the reference, on the device: the next level's grid is set to
    "true" except at its own overwritten points, the refinement adjoint carries the flags
    back (with every band value 1, so a positive sum is the reference's structural
    `Flag` OR), the level's overwritten points read their flag, and the rows whose flag
    survives are kept in order (findall)."""
    lrs = control_points.local_refinements
    if level is None:
        for lev in range(len(lrs) - 2, -1, -1):
            deactivate_overwritten_control_points_(control_points, lev)
        return
    assert 0 <= level <= len(lrs) - 2
    lr, lr_next = lrs[level], lrs[level + 1]
    dev = lr.refinement_values.device
    size_next = tuple(control_points.control_points_refined[level + 1].shape[:-1])
    size_cur = tuple(control_points.control_points_refined[level].shape[:-1])
    nin = len(size_cur)
    flags_next = arrays.ones(size_next + (1,), torch.float64, dev)
    n_next = lr_next.n_refined
    if n_next:
        local_refinement_(flags_next, lr_next.refinement_indices,
                          arrays.zeros((n_next, 1), torch.float64, dev))
    flags_cur = arrays.zeros(size_cur + (1,), torch.float64, dev)
    mult_adjoint_(flags_cur, [A.structure() for A in lr_next.refinement_matrices], flags_next,
                  lr_next.dims_refinement)
    n = lr.n_refined
    if n == 0:
        return
    keep = arrays.zeros((n, 1), torch.float64, dev)
    local_refinement_adjoint_(keep, flags_cur, lr.refinement_indices)
    nout = lr.refinement_values.shape[1]
    dt = lr.refinement_values.dtype
    idx_out = arrays.empty((n, nin), torch.int32, dev)
    vals_out = arrays.empty((n, nout), dt, dev)
    kept = C.c_int64(0)
    _lib.check(_lib.load().sg_select_rows(
        arrays.dtype_code(dt), n, arrays.ptr(keep, "flags"), nin,
        arrays.ptr(lr.refinement_indices, "refinement_indices"), nout,
        arrays.ptr(lr.refinement_values, "refinement_values"), arrays.ptr(idx_out, "indices"),
        arrays.ptr(vals_out, "values"), C.byref(kept), _workspace(n, dev).data_ptr(), _stream()))
    k = int(kept.value)
    new_idx = arrays.empty((k, nin), torch.int32, dev)
    new_idx.copy_(idx_out[:k])
    vals = arrays.empty((k, nout), dt, dev)
    vals.copy_(vals_out[:k])
    lrs[level] = LocalRefinement(lr.dims_refinement, lr.refinement_matrices, new_idx, vals)
