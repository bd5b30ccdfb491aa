"""RefinementMatrix: the reference's banded format (src/refinement_matrix.jl:1-125) and
its set-up algebra (product, collect, identity, dense conversion; :127-363, :447-504).

Refinement matrices are built once at set-up on small sizes, so they live on the host
as numpy arrays in the reference's 1-based format; ``device_arrays`` uploads them for
the library's ``sg_mult`` / ``sg_mult_adjoint``.
"""
from __future__ import annotations

import numpy as np
import torch


class RefinementMatrix:
    """``m x n`` matrix with one contiguous band of nonzeros per row.

    row_pointer[i]: 1-based start of row i in nzval; column_start[i]: 1-based first
    nonzero column of row i.  Rows must satisfy the reference's validity rules
    (validate_refinement_matrix_kernel, src/refinement_matrix.jl:127-181)."""

    def __init__(self, m: int, n: int, row_pointer, column_start, nzval, *, validate=True):
        self.m = int(m)
        self.n = int(n)
        self.row_pointer = np.asarray(row_pointer, dtype=np.int32).copy()
        self.column_start = np.asarray(column_start, dtype=np.int32).copy()
        self.nzval = np.asarray(nzval).copy()
        if not np.issubdtype(self.nzval.dtype, np.floating):
            self.nzval = self.nzval.astype(np.float64)
        assert len(self.row_pointer) == len(self.column_start) == self.m
        assert np.all(np.diff(self.row_pointer) >= 0)
        self._dev = {}
        if validate:
            valid = self.valid_rows()
            if not valid.all():
                bad = [int(i) + 1 for i in np.nonzero(~valid)[0]]
                raise ValueError(f"Invalid rows: {bad}.")

    # ------------------------------------------------------------------ structure
    def row_range(self, i: int):
        """0-based (first column, last column, nzval offset) of row i (0-based)."""
        nxt = len(self.nzval) + 1 if i == self.m - 1 else int(self.row_pointer[i + 1])
        cnt = nxt - int(self.row_pointer[i])
        c0 = int(self.column_start[i]) - 1
        return c0, c0 + cnt - 1, int(self.row_pointer[i]) - 1

    def valid_rows(self) -> np.ndarray:
        """validate_refinement_matrix_kernel (src/refinement_matrix.jl:134-181)."""
        out = np.zeros(self.m, dtype=bool)
        for i in range(self.m):
            c0, c1, _ = self.row_range(i)
            ok = c1 >= c0
            if ok:
                ok = c0 >= 0 and c1 <= self.n - 1
            if i == 0:
                ok = c0 == 0 and self.row_pointer[0] == 1
            if ok and i > 0:
                p0, p1, _ = self.row_range(i - 1)
                ok = p0 <= c0 <= p1 + 1
                if ok:
                    ok = c1 >= p1
            out[i] = ok
        return out

    @property
    def shape(self):
        return (self.m, self.n)

    def size(self):
        return (self.m, self.n)

    def __len__(self):
        return self.m * self.n

    def __getitem__(self, ij):
        i, j = ij
        if not (0 <= i < self.m and 0 <= j < self.n):
            raise IndexError(f"Index ({i + 1}, {j + 1}) out of bounds for refinement matrix of "
                             f"size ({self.m}, {self.n}).")
        c0, c1, z = self.row_range(i)
        return self.nzval[z + j - c0] if c0 <= j <= c1 else self.nzval.dtype.type(0)

    def __eq__(self, other):
        return (isinstance(other, RefinementMatrix) and self.shape == other.shape
                and np.array_equal(self.row_pointer, other.row_pointer)
                and np.array_equal(self.column_start, other.column_start)
                and np.array_equal(self.nzval, other.nzval))

    def collect(self) -> np.ndarray:
        """Dense matrix (collect_refinement_matrix_kernel, src/refinement_matrix.jl:329-363)."""
        out = np.zeros((self.m, self.n), dtype=self.nzval.dtype)
        for i in range(self.m):
            c0, c1, z = self.row_range(i)
            out[i, c0:c1 + 1] = self.nzval[z:z + c1 - c0 + 1]
        return out

    # ------------------------------------------------------------------ product
    def __matmul__(self, B: "RefinementMatrix") -> "RefinementMatrix":
        """C = A * B with the reference's structural product
        (refinement_matrix_mul_nonzeros_kernel and refinement_matrix_multiplication_kernel,
        src/refinement_matrix.jl:183-327): row i of C spans every column that the bands of
        B's rows in A's row-i band cover; values accumulate A[i,k]*B[k,j] in k order."""
        A = self
        if A.n != B.m:
            raise ValueError("Inner dimensions must match")
        dt = np.result_type(A.nzval.dtype, B.nzval.dtype)
        nnz = np.zeros(A.m, dtype=np.int64)
        cs = np.zeros(A.m, dtype=np.int64)
        b_rng = [B.row_range(k) for k in range(B.m)]
        for i in range(A.m):
            a0, a1, _ = A.row_range(i)
            covered = np.zeros(B.n, dtype=bool)
            for k in range(a0, a1 + 1):
                b0, b1, _ = b_rng[k]
                covered[b0:b1 + 1] = True
            cols = np.nonzero(covered)[0]
            nnz[i] = len(cols)
            cs[i] = cols[0] + 1 if len(cols) else 0
        rp = np.ones(A.m, dtype=np.int64)
        rp[1:] = 1 + np.cumsum(nnz[:-1])
        nz = np.zeros(int(nnz.sum()), dtype=dt)
        for i in range(A.m):
            a0, a1, za = A.row_range(i)
            c0 = cs[i] - 1
            for kk, k in enumerate(range(a0, a1 + 1)):
                b0, b1, zb = b_rng[k]
                for j in range(c0, c0 + nnz[i]):
                    if b0 <= j <= b1:
                        nz[rp[i] - 1 + (j - c0)] += A.nzval[za + kk] * B.nzval[zb + j - b0]
        return RefinementMatrix(A.m, B.n, rp, cs, nz)

    __mul__ = __matmul__

    # ------------------------------------------------------------------ conversion
    @classmethod
    def from_dense(cls, A, *, validate=True) -> "RefinementMatrix":
        """RefinementMatrix(::Matrix) (src/refinement_matrix.jl:476-504)."""
        A = np.asarray(A)
        rp, cs, nz = [], [], []
        pointer = 1
        for row in A:
            nzi = np.nonzero(row)[0]
            rp.append(pointer)
            if len(nzi) == 0:
                cs.append(0)
            else:
                cs.append(nzi[0] + 1)
                nz.extend(row[nzi[0]:nzi[-1] + 1])
                pointer += nzi[-1] - nzi[0] + 1
        return cls(A.shape[0], A.shape[1], rp, cs, np.asarray(nz, dtype=A.dtype if
                                                               np.issubdtype(A.dtype, np.floating)
                                                               else np.float64),
                   validate=validate)

    def device_arrays(self, device, dtype: torch.dtype):
        """(row_pointer, column_start, nzval) as CUDA tensors, cached per (device, dtype)."""
        key = (str(device), dtype)
        if key not in self._dev:
            self._dev[key] = (torch.as_tensor(self.row_pointer).to(device),
                              torch.as_tensor(self.column_start).to(device),
                              torch.as_tensor(self.nzval).to(dtype).to(device))
        return self._dev[key]

    def structure(self) -> "RefinementMatrix":
        """The same band with every stored value 1: its adjoint product is positive exactly
        where the reference's structural `Flag` product (src/utils.jl:237-247,
        src/adjoint.jl:117-120) is true."""
        if getattr(self, "_structure", None) is None:
            self._structure = RefinementMatrix(self.m, self.n, self.row_pointer, self.column_start,
                                               np.ones(len(self.nzval)), validate=False)
        return self._structure

    def astype(self, np_dtype) -> "RefinementMatrix":
        return RefinementMatrix(self.m, self.n, self.row_pointer, self.column_start,
                                self.nzval.astype(np_dtype), validate=False)


def rmeye(n: int, *, float_type=np.float32) -> RefinementMatrix:
    """Identity refinement matrix (src/refinement_matrix.jl:447-474)."""
    idx = np.arange(1, n + 1, dtype=np.int32)
    return RefinementMatrix(n, n, idx, idx, np.ones(n, dtype=float_type))


def knot_insertion_matrix(knots_all_old: np.ndarray, degree: int, knot_span_index: int,
                          knot_new) -> RefinementMatrix:
    """RefinementMatrix(spline_dimension, knot_span_index, knot_new)
    (build_refinement_matrix_kernel, src/refinement.jl:1-88): the (n+1) x n matrix that
    writes the old basis in terms of the basis after inserting ``knot_new`` once.
    ``knot_span_index`` is 1-based; arithmetic is in the knots' value type."""
    kn = np.asarray(knots_all_old)
    Tv = kn.dtype.type
    n_basis = len(kn) - degree - 1
    rp = np.zeros(n_basis + 1, dtype=np.int64)
    cs = np.zeros(n_basis + 1, dtype=np.int64)
    nz = np.ones(n_basis + degree + 1, dtype=kn.dtype)
    kv = Tv(knot_new)
    for i in range(1, n_basis + 2):  # 1-based row index
        if i <= knot_span_index - degree:
            rp[i - 1] = i
            cs[i - 1] = i
        elif i <= knot_span_index:
            alpha = (kv - kn[i - 1]) / (kn[i + degree - 1] - kn[i - 1])
            r = 2 * i - knot_span_index + degree - 1
            rp[i - 1] = r
            cs[i - 1] = i - 1
            nz[r - 1] = Tv(1) - alpha
            nz[r] = alpha
        else:
            rp[i - 1] = i + degree
            cs[i - 1] = i - 1
    return RefinementMatrix(n_basis + 1, n_basis, rp, cs, nz)


def insert_knot_values(knot_values: np.ndarray, multiplicities: np.ndarray, knot_new):
    """Host part of insert_knot(knot_vector, knot_new) (src/refinement.jl:90-133): the new
    knot values and multiplicities with ``knot_new`` (multiplicity 1) and the 1-based
    knot span index ``sum(multiplicities[1:pos-1])`` of the insertion."""
    kv = np.asarray(knot_values)
    mult = np.asarray(multiplicities, dtype=np.int32)
    kn = kv.dtype.type(knot_new)
    assert not np.any(kv == kn)
    pos = int(np.searchsorted(kv, kn, side="left"))  # searchsortedfirst(kv, kn) - 1
    return np.insert(kv, pos, kn), np.insert(mult, pos, 1), int(mult[:pos].sum())


def expand_knots(knot_values: np.ndarray, multiplicities: np.ndarray) -> np.ndarray:
    """knots_all on the host (the expansion the device does in sg_expand_knots)."""
    return np.repeat(np.asarray(knot_values), np.asarray(multiplicities, dtype=np.int64))


def knot_span_sequence(knot_values, multiplicities, knots_new=None):
    """The knot bookkeeping of refine(::SplineDimension; knots_new)
    (src/refinement.jl:256-284): insert every knot (default: the midpoints of the knot
    spans, in the knots' value type) in order.  Returns (values, multiplicities, the
    inserted knots, the 1-based knot span index of each at its insertion)."""
    kv = np.asarray(knot_values)
    mult = np.asarray(multiplicities, dtype=np.int32)
    if knots_new is None:
        knots_new = kv[:-1] + np.diff(kv) / kv.dtype.type(2)
    knots = np.asarray(knots_new, dtype=kv.dtype)
    spans = []
    for k in knots:
        kv, mult, ksi = insert_knot_values(kv, mult, k)
        spans.append(ksi)
    return kv, mult, knots, spans


def refine_knots(knot_values, multiplicities, degree: int, knots_new=None):
    """Host part of refine(::SplineDimension; knots_new) (src/refinement.jl:237-284): insert
    every knot (default: the midpoints of the knot spans, in the knots' value type) and
    compose the refinement matrices, ``R = R_knot * R``.  Returns (values, multiplicities,
    R)."""
    kv = np.asarray(knot_values)
    mult = np.asarray(multiplicities, dtype=np.int32)
    if knots_new is None:
        knots_new = kv[:-1] + np.diff(kv) / kv.dtype.type(2)
    n_basis = int(mult.sum()) - degree - 1
    R = rmeye(n_basis, float_type=kv.dtype)
    for k in np.asarray(knots_new, dtype=kv.dtype):
        knots_old = expand_knots(kv, mult)
        kv, mult, ksi = insert_knot_values(kv, mult, k)
        R = knot_insertion_matrix(knots_old, degree, ksi, k) @ R
    return kv, mult, R
