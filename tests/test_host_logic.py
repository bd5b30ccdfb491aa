"""Host logic of the package (no GPU): refinement-matrix algebra (the reference's
test/test_refinement_matrix.jl), knot insertion, Julia-layout helpers, validation
messages, and the C-ABI library's export table."""
import os
import re

import numpy as np
import pytest

import splinegrids as sg
from conftest import ROOT


def test_unit_matrix():
    """test/test_refinement_matrix.jl:16-37."""
    N = 100
    M = sg.rmeye(N)
    assert M[24, 24] == 1 and M[24, 25] == 0
    with pytest.raises(IndexError, match=r"Index \(101, 1\) out of bounds for refinement matrix "
                                         r"of size \(100, 100\)\."):
        M[N, 0]
    M2 = M @ M
    assert M2 == M and M2.shape == (N, N) and len(M2) == N * N


def test_diagonal_product():
    """test/test_refinement_matrix.jl:39-48."""
    rng = np.random.default_rng(1)
    A = sg.RefinementMatrix.from_dense(np.diag(rng.random(100)))
    B = sg.RefinementMatrix.from_dense(np.diag(rng.random(100)))
    assert np.array_equal((A @ B).nzval, A.nzval * B.nzval)


def _banded(m, n, lo, hi, rng):
    A = rng.random((m, n))
    i, j = np.indices((m, n))
    A[(j < i - lo) | (j > i + hi)] = 0
    return A


def test_banded_product_matches_dense():
    """test/test_refinement_matrix.jl:50-61 (brand(100,100,4,3) * brand(100,200,3,5))."""
    rng = np.random.default_rng(1)
    A = sg.RefinementMatrix.from_dense(_banded(100, 100, 4, 3, rng))
    B = sg.RefinementMatrix.from_dense(_banded(100, 200, 3, 5, rng))
    assert np.allclose((A @ B).collect(), A.collect() @ B.collect(), rtol=1e-12)


def test_invalid_rows_messages():
    """test/test_refinement_matrix.jl:63-75."""
    M = np.zeros((2, 50))
    M[0, :20] = 1
    M[1, 38:] = 1
    with pytest.raises(ValueError, match=re.escape("Invalid rows: [2].")):
        sg.RefinementMatrix.from_dense(M)
    M = np.zeros((3, 50))
    M[0, :25] = 1
    M[2, 25:] = 1
    with pytest.raises(ValueError, match=re.escape("Invalid rows: [2, 3].")):
        sg.RefinementMatrix.from_dense(M)


def test_validation_agrees_with_oracle(oracle):
    rng = np.random.default_rng(7)
    for _ in range(50):
        A = _banded(12, 15, 2, 3, rng)
        A[rng.random(A.shape) < 0.1] = 0
        R = sg.RefinementMatrix.from_dense(A, validate=False)
        v = oracle.validate_refinement_matrix(R.row_pointer, R.column_start, len(R.nzval), R.n)
        assert np.array_equal(v, R.valid_rows())


def test_knot_insertion_matrix_reproduces_basis(oracle):
    """Inserting a knot: old basis = R' new basis at every sample (FP64)."""
    kv = np.array([0.0, 0.2, 0.5, 0.7, 1.0])
    mult = np.array([4, 1, 1, 1, 4], dtype=np.int32)
    deg = 3
    knots = sg.expand_knots(kv, mult)
    kv2, mult2, ksi = sg.insert_knot_values(kv, mult, 0.33)
    R = sg.knot_insertion_matrix(knots, deg, ksi, 0.33)
    knots2 = sg.expand_knots(kv2, mult2)
    t = np.linspace(0, 1, 101)
    def dense(kn):
        si = oracle.sample_indices(t, kn, deg)
        b = oracle.basis(kn, t, si, deg, 0)
        return oracle.decompress(b, si, deg, 0, len(kn) - deg - 1)
    assert np.allclose(dense(knots), dense(knots2) @ R.collect(), atol=1e-14)


def test_colmajor_helpers():
    import torch
    t = sg.arrays.zeros((3, 4, 2), torch.float64, "cpu")
    assert sg.arrays.is_colmajor(t) and t.stride() == (1, 3, 12)
    t[1, 2, 1] = 5
    flat = sg.arrays.vec(t)
    assert flat[1 + 3 * 2 + 12 * 1] == 5
    back = sg.arrays.reshape(flat, (3, 4, 2))
    assert back[1, 2, 1] == 5


def test_derivative_order_messages(caplog):
    class D:
        max_derivative_order = 1
    with pytest.raises(ValueError, match=re.escape(
            "Invalid derivative order(s) supplied. If you want to evaluate (higher order) "
            "derivatives, specify this at construction as SplineDimension(...; "
            "max_derivative_order).")):
        sg.validate_partial_derivatives([D(), D()], (2, 1))
    msgs = [r.getMessage() for r in caplog.records]
    assert msgs == ["The maximum derivative order available for spline dimension 1 is 1, got 2."]


def _header_functions():
    src = open(os.path.join(ROOT, "include", "splinegrids_b200.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(sg_[a-z_0-9]+)\s*\(",
                                 src, flags=re.M)))


def test_library_exports_every_declared_symbol():
    """The C-ABI library loads (no GPU needed) and exports every function the header
    declares; the ctypes table declares the same set."""
    import build as sg_build
    path = sg_build.build()
    import ctypes
    lib = ctypes.CDLL(path)
    names = _header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    from splinegrids import _lib
    assert sorted(_lib.SIGNATURES) == names


@pytest.mark.parametrize("m,n,damp", [(60, 20, 0.0), (60, 20, 0.3), (200, 50, 0.0),
                                      (80, 30, 0.0)])
def test_oracle_lsqr_matches_scipy(oracle, m, n, damp):
    """The oracle's LSQR (the checker of the device solver) against scipy's implementation
    of the same published algorithm (Paige & Saunders 1982), with IterativeSolvers'
    defaults: same stop code, iteration count and solution."""
    sl = pytest.importorskip("scipy.sparse.linalg")
    rng = np.random.default_rng(m + n)
    A = rng.standard_normal((m, n))
    b = rng.standard_normal(m)
    x, istop, itn, info = oracle.lsqr(lambda v: A @ v, lambda u: A.T @ u, b, n, damp=damp)
    eps = np.finfo(np.float64).eps
    r = sl.lsqr(A, b, damp=damp, atol=np.sqrt(eps), btol=np.sqrt(eps), conlim=1 / np.sqrt(eps),
                iter_lim=max(m, n))
    assert (istop, itn) == (r[1], r[2])
    assert np.abs(x - r[0]).max() <= 1e-10 * np.abs(r[0]).max()
    assert info["acond"] == pytest.approx(r[6], rel=1e-8)
    # consistent system: recovers the solution
    xt = rng.standard_normal(n)
    x2, istop2, _, _ = oracle.lsqr(lambda v: A @ v, lambda u: A.T @ u, A @ xt, n)
    assert istop2 in (1, 2) and np.abs(x2 - xt).max() <= 1e-6


def test_knot_span_sequence_matches_composed_insertions():
    """The host bookkeeping of the device refinement: the spans it hands to
    sg_refine_matrix are those refine_knots uses knot by knot, and the final knot vector
    is the same."""
    kv = np.array([0.0, 0.2, 0.5, 1.0])
    mult = np.array([4, 1, 2, 4], np.int32)
    kv2, mult2, knots, spans = sg.knot_span_sequence(kv, mult)
    kv3, mult3, R = sg.refine_knots(kv, mult, 3)
    assert np.array_equal(kv2, kv3) and np.array_equal(mult2, mult3)
    assert np.allclose(knots, [0.1, 0.35, 0.75])
    # span = number of expanded knots below the inserted knot, at its insertion
    cur_v, cur_m = kv, mult
    for k, s in zip(knots, spans):
        assert s == int(np.sum(sg.expand_knots(cur_v, cur_m) < k))
        cur_v, cur_m, _ = sg.insert_knot_values(cur_v, cur_m, k)
    assert R.m == int(mult2.sum()) - 4 and R.n == int(mult.sum()) - 4


def test_pipeline_chunks_balance_output_sizes():
    """GridBatchPipeline cuts the grids into consecutive chunks of about equal output
    size, never empty, at most n_chunks."""
    from splinegrids.batch import chunk_ranges
    assert chunk_ranges([5, 1, 1, 1, 8, 2, 2, 4], 3) == [(0, 4), (4, 5), (5, 8)]
    assert chunk_ranges([1] * 10, 4) == [(0, 3), (3, 5), (5, 8), (8, 10)]
    assert chunk_ranges([7], 8) == [(0, 1)]
    r = chunk_ranges([3, 9, 1, 1, 1, 1, 20], 16)
    assert r[0][0] == 0 and r[-1][1] == 7 and all(b > a for a, b in r)
    assert all(r[i][1] == r[i + 1][0] for i in range(len(r) - 1))


def test_batched_workload_size_is_the_benchmarked_one():
    """The batched configuration's draws (host only) give the values per step and the
    algorithmic bytes that the benchmark reports (256 grids, 16 sets, FP32)."""
    import bench
    specs = bench.batched_specs()
    assert len(specs) == 256
    fwd, adj, vals = bench.batched_bytes(specs)
    assert vals == 2503130672
    assert all(8 <= min(s["n_cp"]) and max(s["n_cp"]) <= 128 for s in specs)
    assert all(64 <= min(s["ns"]) and max(s["ns"]) <= 1024 for s in specs)
    assert all(s["deg"] in (1, 2, 3) and s["ch"] in (16, 48) for s in specs)
    # forward + adjoint algorithmic bytes: the eval write and the cotangent read dominate
    assert 2 * vals * 4 < fwd + adj < 2.1 * vals * 4



def test_benchmarked_pipeline_sub_batches_are_balanced():
    """The e2e pipeline's 16 sub-batches over the benchmarked 256 grids: consecutive,
    none empty, each within one grid's output of the mean (so no sub-batch's upload or
    download holds the others back)."""
    import bench
    from splinegrids.batch import chunk_ranges
    specs = bench.batched_specs()
    sizes = [s["ns"][0] * s["ns"][1] * s["ch"] for s in specs]
    r = chunk_ranges(sizes, 16)
    assert len(r) == 16 and r[0][0] == 0 and r[-1][1] == len(sizes)
    assert all(r[i][1] == r[i + 1][0] for i in range(len(r) - 1))
    per = [sum(sizes[a:b]) for a, b in r]
    mean = sum(sizes) / 16
    assert max(per) <= mean + max(sizes) and min(per) >= mean - max(sizes)
